"""Benchmark: per-snapshot Tree-SVD refresh on one GB300 (or N replicas).

A step is one snapshot refresh of the named workload: insert the delta's
edges, refresh + push PPR (forward and reverse for directed graphs), log
transform + lazy test of every column block, frPCA of the dirty blocks, merge
of their ancestors. The first snapshot (pushed from scratch) is set-up and is
not timed; the timed steps are later, dynamic snapshots. The default workload
is the precision configuration's graph (directed R-MAT, N = 6,216,199,
M = 177,862,656, |S| = 3000, 128 blocks, d = 128) refreshed by 1 %-insertion
snapshots (1.78M edges each) after a 70 % first snapshot.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is inserted edges per second with every delta resident in HBM before
the timed region; `e2e` is the same metric through tsvd_session_step with the
deltas in pinned host memory (copied in every step) and the |S| x d embedding
read back every step, on the deltas that follow the timed ones in the same
session (at most K of them). p50/p99 are per-snapshot latencies.

--impl reference times the reference's own CPU code for the path on the host
cores (its graph insert, dense-path refresh and push, log transform and lazy
test, compiled from its sources into oracle/_ref/; its frpca.c and merge SVD
over an MKL stand-in): each step is one dynamic snapshot for a sample of
sources, timed whole (`ms_per_step`), and scaled to the full snapshot in the
metric's unit (`value`, with the scaled seconds beside it). Its inputs come
from the oracle's own generator (the same bytes), so that process never
loads this library.

Multi-GPU: the path is replicated, not sharded (one independent session per
rank, no collective on the data path); value = all ranks' inserted edges per
second over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "tree-embedding_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "p50/p99 re-embed latency & edge updates/s, 1 GB300, vs plain GPU form"
DEFAULT_WORKLOAD = "rmat-d-6.2m-1pct"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--sources", type=int, default=None)
    ap.add_argument("--parts", type=int, default=None)
    ap.add_argument("--snapshots", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--hierarchy", type=int, default=None,
                    help="merge arity (the workload's default is 2; the reference's run.sh uses 8)")
    ap.add_argument("--host-reserve", default="auto", choices=["auto", "on", "off"],
                    help="PPR reserve in pinned host memory (auto: as the workload says)")
    ap.add_argument("--pipelined", action="store_true",
                    help="time tsvd_session_run (factor stage of snapshot k overlapped with the "
                         "push of k+1: more snapshots/s, longer per-snapshot latency) instead of "
                         "one tsvd_session_step per snapshot")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain-GPU-form leg (same session, the deltas after the e2e leg)")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--cpu-sources", type=int, default=None,
                    help="sources in the CPU sample (default: two per host thread)")
    ap.add_argument("--seed", type=int, default=20231)
    ap.add_argument("--push-levels", type=int, default=None,
                    help="threshold schedule levels of the push (default: the library's)")
    ap.add_argument("--push-ratio", type=float, default=None)
    ap.add_argument("--push-hub-degree", type=int, default=None,
                    help="apply the threshold schedule to vertices of at least this degree only")
    ap.add_argument("--push-cofrac", type=float, default=None,
                    help="co-push residues above this fraction of rmax on runs being pushed")
    ap.add_argument("--serve", action="store_true",
                    help="serving measurement instead of the headline: tenants of different sizes "
                         "on one GPU, Poisson-arriving edge batches, p50/p99 request latency")
    ap.add_argument("--serve-tenants", type=int, default=8)
    ap.add_argument("--serve-requests", type=int, default=160)
    ap.add_argument("--serve-slots", type=int, default=4)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device),
                                      "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, nm in enumerate(names):
                if len(s) > 4 + i and s[4 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def workload(args, generator=None):
    import workloads as W
    cfg = W.scaled(args.workload, n=args.n, m=args.m, sources=args.sources,
                   n_parts=args.parts, snapshots=args.snapshots)
    if args.hierarchy:
        cfg["hierarchy_n"] = args.hierarchy
    need = 1 + args.warmup + args.steps
    if cfg["snapshots"] < need:
        raise SystemExit("workload %s has %d deltas; --warmup + --steps (%d) must not exceed them "
                         "(or pass --snapshots)" % (args.workload, cfg["snapshots"] - 1, need - 1))
    edges, snaps, sources = W.build(cfg, seed=args.seed, generator=generator)
    return cfg, snaps, sources


def host_reserve(args, cfg):
    return {"on": True, "off": False}.get(args.host_reserve, bool(cfg.get("host_reserve")))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ------------------------------------------------------------------ our arm
def run_ours(args, cfg, snaps, sources, device):
    """Our arm. Each timed snapshot is one tsvd_session_step_device call (or,
    with --pipelined, all K go through one tsvd_session_run_device call).
    Every snapshot is complete (embedding written) inside the timed region.
    Per-snapshot latency (stats ms_total) runs from the start of a snapshot's
    insert to the end of its factor stage. The e2e leg continues the same
    session through tsvd_session_step with host deltas, then the plain-form
    leg on the deltas after those."""
    import torch
    import tsvd_gb300 as T
    import workloads as W

    torch.cuda.set_device(device)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw["device"] = device
    kw["seed"] = args.seed
    kw["ppr_host_reserve"] = host_reserve(args, cfg)
    for key in ("push_levels", "push_ratio", "push_hub_degree", "push_cofrac"):
        if getattr(args, key) is not None:
            kw[key] = getattr(args, key)
    t0i, t1i = 1 + args.warmup, 1 + args.warmup + args.steps
    timed = snaps[t0i:t1i]
    off = np.concatenate([[0], np.cumsum([len(e) for e in timed])]).astype(np.int64)
    dev = [torch.from_numpy(np.ascontiguousarray(e)).to(f"cuda:{device}") for e in snaps[:t0i]]
    dev_timed = torch.from_numpy(np.ascontiguousarray(np.concatenate(timed))).to(f"cuda:{device}")
    res = {"push_schedule": {k: kw.get(k, d) for k, d in
                             (("push_levels", 1), ("push_ratio", 8.0), ("push_hub_degree", 0),
                              ("push_cofrac", 0.85))}}
    with T.Session(cfg["n"], sources, **kw) as s:
        t = time.perf_counter()
        s.step_device(dev[0].data_ptr(), len(snaps[0]))  # set-up: first snapshot, from scratch
        res["setup_s"] = time.perf_counter() - t
        for k in range(args.warmup):
            s.step_device(dev[1 + k].data_ptr(), len(snaps[1 + k]))
        stream = torch.cuda.ExternalStream(s.stream(), device=device)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = T.launch_count()
        torch.cuda.synchronize(device)
        with ClockSampler(device) as clk:
            torch.cuda.nvtx.range_push("timed")  # profilers can select the timed launches
            ev0.record(stream)
            t0 = time.perf_counter()
            if args.pipelined:
                stage, _ = s.run_device(dev_timed.data_ptr(), off, embeddings=False)
            else:
                stage = []
                for k in range(args.steps):
                    s.step_device(dev_timed.data_ptr() + int(off[k]) * 8, int(off[k + 1] - off[k]))
                    stage.append(s.stats())
            ev1.record(stream)  # after the calls returned: every snapshot is complete
            torch.cuda.synchronize(device)
            wall = time.perf_counter() - t0
            torch.cuda.nvtx.range_pop()
        launches = T.launch_count() - launches0
        ms = ev0.elapsed_time(ev1)
        res.update(ms=ms, wall=wall, per_step=[st["ms_total"] for st in stage], stages=stage,
                   launches=launches, clocks=clk.summary(), edges=int(off[-1]))
        del dev, dev_timed
        left = snaps[t1i:]
        n_plain = 0 if args.no_plain else min(args.plain_steps, len(left) // 2)
        rest = left[:min(args.steps, len(left) - n_plain)]
        plain_snaps = left[len(rest):len(rest) + n_plain]
        if not args.no_e2e and rest:
            res.update(e2e_leg(s, rest, sources, cfg, device, stream))
        if plain_snaps:
            res["plain"] = plain_leg(s, plain_snaps, device, stream)
    return res


def e2e_leg(s, rest, sources, cfg, device, stream):
    """End to end through the C-ABI on the deltas that follow the timed ones:
    host pairs (pinned) copied in and the embedding read back every step."""
    import ctypes

    import torch
    import tsvd_gb300 as T
    pinned = [torch.from_numpy(np.ascontiguousarray(e)).pin_memory() for e in rest]
    L = T.lib()
    emb = np.zeros((len(rest), len(sources), cfg["rank_d"]), np.float64)
    stats = (T.StepStats * len(rest))()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    i32p, f64p = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
    ev0.record(stream)
    for k, e in enumerate(pinned):
        T._check(L.tsvd_session_step(s._h, ctypes.cast(e.data_ptr(), i32p), len(rest[k])))
        T._check(L.tsvd_session_embedding(s._h, emb[k].ctypes.data_as(f64p)))
        T._check(L.tsvd_session_last_stats(s._h, ctypes.byref(stats[k])))
    ev1.record(stream)
    torch.cuda.synchronize(device)
    assert np.isfinite(emb).all()
    edges = int(sum(len(e) for e in rest))
    return {"e2e_ms": ev0.elapsed_time(ev1), "e2e_edges": edges, "e2e_steps": len(rest),
            "e2e_lat": [stats[k].ms_total for k in range(len(rest))],
            "h2d": int(edges * 8 / len(rest)), "d2h": int(len(sources) * cfg["rank_d"] * 8)}


def plain_leg(s, plain_snaps, device, stream):
    """The same session switched to the plain GPU form for the next deltas
    (device-resident, one tsvd_session_step_device each): per-snapshot
    latency of the form the mixed-precision batched form is measured
    against."""
    import torch
    import tsvd_gb300 as T
    dev = [torch.from_numpy(np.ascontiguousarray(e)).to(f"cuda:{device}") for e in plain_snaps]
    s.set_form(T.FORM_PLAIN)
    stages = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    ev0.record(stream)
    for e, d in zip(plain_snaps, dev):
        s.step_device(d.data_ptr(), len(e))
        stages.append(s.stats())
    ev1.record(stream)
    torch.cuda.synchronize(device)
    s.set_form(T.FORM_MIXED)
    lat = [st["ms_total"] for st in stages]
    edges = int(sum(len(e) for e in plain_snaps))
    return {"steps": len(stages), "ms": ev0.elapsed_time(ev1), "edges": edges, "lat": lat,
            "stages": stages}


# ------------------------------------------------------------- CPU samples
class _QuietStdout:
    """The reference's graph reader reports progress on stdout; keep it off
    the bench's one-line output (fd 1 goes to /dev/null meanwhile)."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *a):
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def cpu_sample(cfg, snaps, sources, steps, k=None, threads=None, budget_s=150.0):
    """Times the reference's own CPU code on a bounded sample of the workload.

    Set-up (untimed): the reference graph store is fed the first snapshot
    through its own reader, and k sampled sources are pushed from scratch
    (both directions for a directed graph). Each step then times one dynamic
    snapshot: the reference's insert of the delta file, its refresh + push for
    the k sources (std::threads over source ranges, as its drivers run them),
    its log transform + lazy test of every block on those k rows, frPCA
    (frpca.c) of two real blocks of the snapshot (the k sampled rows tiled to
    |S| rows, so the block has the full shape, density and values), and one
    merge SVD of their two factors. The full snapshot is the sum of the
    insert, (push + log) x |S|/k, frPCA x blocks (every block dirty) and the
    merge x (blocks - 1).

    With oracle/_ref absent (no reference sources were ever staged), the
    oracle's restatement (oracle/) stands in for each piece."""
    from oracle import native
    from oracle.tree_oracle import frpca as port_frpca
    from oracle.tree_oracle import gaussian_matrix, log_transform
    import scipy.sparse as sp

    threads = threads or os.cpu_count() or 1
    S, n, nparts = len(sources), cfg["n"], cfg["n_parts"]
    k = min(S, k or 2 * threads)
    sub = np.sort(np.random.default_rng(0).choice(sources, k, replace=False)).astype(np.int32)
    alpha, rmax, d, q = cfg["alpha"], cfg["rmax"], cfg["rank_d"], cfg["passes_q"]
    dirs = 2 if cfg["directed"] else 1
    cd = n // nparts
    kind = "reference" if native.ref_available() else "port"
    kind_frpca = "reference" if native.ref_frpca_available() else "port"
    tmp = tempfile.mkdtemp(prefix="tsvd_cpu_")
    t_setup = time.perf_counter()
    if kind == "reference":
        path0 = os.path.join(tmp, "snap0.txt")
        native.write_edges_text(path0, snaps[0])
        g = native.RefGraph(n, cfg["directed"])
        with _QuietStdout():
            g.insert_file(path0)
        os.unlink(path0)
        st = [native.RefPPR(n, sub, nparts, alpha, rmax) for _ in range(dirs)]
        for dd in range(dirs):
            st[dd].step(g, dd, 1, 2, threads)
    else:
        g = native.OracleGraph(n, cfg["directed"])
        g.insert(snaps[0])
        st = [native.OraclePPR(n, sub) for _ in range(dirs)]
        for dd in range(dirs):
            st[dd].refresh(g, dd, 1, 2, alpha, rmax, threads=threads)
            st[dd].push(g, dd, alpha, rmax, threads=threads)
    t_setup = time.perf_counter() - t_setup
    out = []
    t_budget = time.perf_counter()
    for step in range(steps):
        delta = snaps[1 + step]
        path = os.path.join(tmp, "delta.txt")
        if kind == "reference":
            native.write_edges_text(path, delta)
        w0 = time.perf_counter()
        if kind == "reference":
            with _QuietStdout():
                g.insert_file(path)
        else:
            g.insert(delta)
        t_ins = time.perf_counter() - w0
        t = time.perf_counter()
        for dd in range(dirs):
            if kind == "reference":
                st[dd].step(g, dd, 2 + step, 2, threads)
            else:
                st[dd].refresh(g, dd, 2 + step, 2, alpha, rmax, threads=threads)
                st[dd].push(g, dd, alpha, rmax, threads=threads)
        t_push = time.perf_counter() - t
        t = time.perf_counter()
        blocks = []
        if kind == "reference":
            st[0].log_only(2 + step, cfg.get("delta", 0.3), np.zeros(nparts))
            for b in (0, nparts // 2):
                rp, ci, va = st[0].block_csr(b)
                width = n - (nparts - 1) * cd if b == nparts - 1 else cd
                blocks.append(sp.csr_matrix((va, ci, rp), shape=(k, width)))
        else:
            p = st[0].reserve().astype(np.float64)
            for b in range(nparts):
                c1 = n if b == nparts - 1 else (b + 1) * cd
                A = log_transform(p[:, b * cd:c1], rmax, cfg["transform"], n)
                if b in (0, nparts // 2):
                    blocks.append(sp.csr_matrix(A))
        t_log = time.perf_counter() - t
        # frPCA of two real blocks at full |S|: the k rows tiled
        t_fr, factors = [], []
        for A in blocks:
            full = sp.vstack([A] * (S // k + 1), format="csr")[:S]
            t = time.perf_counter()
            if kind_frpca == "reference":
                U, Sg, V, _ = native.ref_frpca(full, d, q, seed=7)
                Sg = Sg[::-1]
                U = U[:, ::-1]
            else:
                omega = gaussian_matrix(7, 0, full.shape[1], d + 5)
                U, Sg, V = port_frpca(full, d, q, omega=omega)
                Sg, U = Sg[::-1], U[:, ::-1]
            t_fr.append(time.perf_counter() - t)
            factors.append(U * Sg[None, :])
        M = np.hstack(factors)
        t = time.perf_counter()
        if kind_frpca == "reference":
            native.ref_merge_svd(M, d)
        else:
            np.linalg.svd(M, full_matrices=False)
        t_merge = time.perf_counter() - t
        wall = time.perf_counter() - w0
        scaled = t_ins + (t_push + t_log) * S / k + float(np.mean(t_fr)) * nparts + \
            t_merge * (nparts - 1)
        out.append(dict(wall_s=wall, scaled_s=scaled, edges=len(delta), insert_s=t_ins,
                        push_s=t_push, log_s=t_log, frpca_block_s=float(np.mean(t_fr)),
                        merge_s=t_merge))
        if time.perf_counter() - t_budget > budget_s:
            break
    try:
        os.rmdir(tmp)
    except OSError:
        pass
    desc = ("%s code on %d host threads: one dynamic snapshot per step (%d-edge deltas): insert "
            "of the delta file; refresh + push of %d of %d sources (%s), x %.1f; log transform + "
            "lazy test of all %d blocks on those rows, x %.1f; frPCA (q = %d, d = %d) of two real "
            "%d x %d blocks (the sampled rows tiled to |S| rows; %s), x %d blocks (all assumed "
            "dirty); one %d x %d merge SVD, x %d. Set-up (first snapshot, from-scratch push of "
            "the sampled sources) %.0f s, untimed" % (
                "the reference's own" if kind == "reference" else "the oracle's restated",
                threads, len(snaps[1]), k, S, "forward and reverse" if dirs == 2 else "undirected",
                S / k, nparts, S / k, q, d, S, cd, kind_frpca + " frpca.c" if kind_frpca ==
                "reference" else "oracle frPCA", nparts, S, 2 * d, nparts - 1, t_setup))
    return {"steps": out, "threads": threads, "kind": kind, "sample": desc, "k": k,
            "setup_s": t_setup}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import native
    cfg, snaps, sources = workload(args, generator=native)
    info = cpu_sample(cfg, snaps, sources, steps=max(1, args.steps), k=args.cpu_sources)
    st = info["steps"]
    rate = [s["edges"] / s["scaled_s"] for s in st]
    v = float(statistics.median(rate))
    scaled_ms = [s["scaled_s"] * 1e3 for s in st]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "edge updates/s",
            "n_gpus": args.gpus, "steps": len(st), "warmup": 0,
            "ms_per_step": float(np.mean([s["wall_s"] for s in st]) * 1e3),
            "p50_ms": float(np.percentile(scaled_ms, 50)),
            "p99_ms": float(np.percentile(scaled_ms, 99)),
            "scaled_ms_per_snapshot": float(np.mean(scaled_ms)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 PPR state, f64 arithmetic (reference dense path); f64 frPCA and merge",
            "data": "synthetic (seeded R-MAT from the oracle's generator)",
            "config": {"workload": cfg["name"], "n": cfg["n"], "m": cfg["m"],
                       "sources": cfg["sources"], "n_parts": cfg["n_parts"],
                       "rank_d": cfg["rank_d"], "snapshots": cfg["snapshots"]},
            "stage_s_mean": {k: float(np.mean([s[k] for s in st]))
                             for k in ("insert_s", "push_s", "log_s", "frpca_block_s", "merge_s")},
            "cpu_baseline": {"value": v, "unit": "edge updates/s", "cores": info["threads"],
                             "kind": info["kind"], "sample": info["sample"]},
            "e2e": {"value": v, "unit": "edge updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# --------------------------------------------------------------- roofline
def push_roofline(stages):
    """Roofline of the dominant kernels (push_kernel + push_heavy_kernel) over
    the timed steps, duration from CUDA events around every launch on the
    session stream.

    `achieved` counts the bytes of the reference's FIFO push at the width the
    state is stored in (fp32 residue and reserve): per executed push of (v, s)
    4 (r_v read) + 4 (r_v write) + 8 (p_v read-modify-write) + 8 (row offsets),
    and per edge update 4 (neighbour id) + 8 (r_u read-modify-write).

    `achieved_min` counts the bytes this design has to move at least: per lane
    push 16 (fp32 residue exchange + reserve update), per lane edge update 8
    (fp32 atomic read-modify-write), per item-neighbour 4 (the neighbour id is
    read once for the 64 sources of a chunk), per item 20 (frontier entry, row
    start, degree)."""
    pk, _ = peaks()
    peak = float(pk.get("hbm_gbs", 6800.0))
    pushes = sum(s["pushes"] for s in stages)
    upd = sum(s["push_edge_updates"] for s in stages)
    items = sum(s["push_items"] for s in stages)
    iedges = sum(s["push_item_edges"] for s in stages)
    ms = sum(s["ms_push_kernels"] for s in stages)
    launches = sum(2 * s["push_rounds"] for s in stages)
    byts = 24.0 * pushes + 12.0 * upd
    byts_min = 16.0 * pushes + 8.0 * upd + 4.0 * iedges + 20.0 * items
    sec = ms / 1e3
    achieved = byts / sec / 1e9 if ms > 0 else 0.0
    achieved_min = byts_min / sec / 1e9 if ms > 0 else 0.0
    return {"kernel": "push_kernel+push_heavy_kernel", "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "traffic_note": TRAFFIC_NOTE,
            "algorithmic_bytes_per_launch": byts / max(1, launches),
            "achieved_min": achieved_min, "frac_min": achieved_min / peak,
            "min_bytes_per_launch": byts_min / max(1, launches),
            "launches": launches, "kernel_ms": ms,
            "lanes_per_item": pushes / max(1, items),
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth), of measured"}


# DRAM counters are only captured on cases of a few GB. The push's traffic
# per item-neighbour depends on how many reductions a residue run receives
# per round (its L2 reuse), which differs between such a case and the
# full-size state, so a small-case figure does not scale to this launch.
TRAFFIC_NOTE = ("not measured at this size: DRAM counters are captured on cases of a few GB "
                "only, and the push's DRAM bytes per item-neighbour depend on the reductions "
                "a residue run receives per round, which do not scale from such a case")


def tail_attribution(stages):
    """Where the slowest snapshots spend their extra time: per stage, the mean
    over the steps at or above the 90th latency percentile minus the median
    over all steps, with the push work counters that explain the push part."""
    lat = np.array([s["ms_total"] for s in stages])
    if len(lat) < 2:
        return None
    slow = lat >= np.percentile(lat, 90)
    keys = ("ms_insert", "ms_push", "ms_log", "ms_frpca", "ms_merge")
    out = {"slow_steps": int(slow.sum()),
           "extra_ms": {k: float(np.mean([s[k] for s, f in zip(stages, slow) if f]) -
                                 np.median([s[k] for s in stages])) for k in keys}}
    for k in ("push_rounds", "push_item_edges", "dirty_blocks"):
        med = float(np.median([s[k] for s in stages]))
        out[k + "_ratio"] = float(np.mean([s[k] for s, f in zip(stages, slow) if f])) / max(med, 1)
    return out


def aggregate(ms, edges, device=None):
    """Whole-job throughput of independent replicas: every rank's edges over
    the slowest rank's time (max over ranks; identity without a process group)."""
    import torch
    import torch.distributed as tdist
    world = tdist.get_world_size() if tdist.is_available() and tdist.is_initialized() else 1
    if world > 1:
        t = torch.tensor([float(ms), float(edges)], dtype=torch.float64,
                         device=device if device is not None else "cpu")
        mx = t.clone()
        tdist.all_reduce(mx, op=tdist.ReduceOp.MAX)
        tot = t.clone()
        tdist.all_reduce(tot, op=tdist.ReduceOp.SUM)
        ms, edges = float(mx[0].item()), float(tot[1].item())
    return ms, edges, edges / (ms / 1e3)


def run_serve(args):
    """Serving form on one GPU: `--serve-tenants` directed R-MAT tenants with
    N log-spaced in [1e5, 3e6] (M = 10 N), |S| in [500, 2000], d in {64, 128},
    each admitted by its HBM footprint and set up with half of its edges;
    then `--serve-requests` edge batches with sizes log-uniform in
    [1e3, min(1e5, M / 40)] drawn from the tenants' remaining edges arrive as
    a Poisson stream (mean gap 30 ms) at random tenants, each followed by an
    embedding query. Reports p50 / p99 latency (arrival to completion) of the
    updates, edge updates per second over the stream, and the mean service
    time per tenant size."""
    import torch
    import tsvd_gb300 as T
    import workloads as W
    rng = np.random.default_rng(args.seed)
    device = 0
    torch.cuda.set_device(device)
    k = args.serve_tenants
    ns = np.unique(np.round(np.logspace(5, np.log10(3e6), k)).astype(int))
    tenants = []
    with T.Server(device=device, slots=args.serve_slots) as srv:
        t_setup = time.perf_counter()
        for i, n in enumerate(ns):
            cfg = W.scaled("rmat-d-2.7m", n=int(n), m=int(10 * n),
                           sources=int(rng.integers(500, 2001)), n_parts=16,
                           rank_d=int(rng.choice([64, 128])), snapshots=2)
            _, snaps, src = W.build(cfg, seed=args.seed + i)
            kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
            try:
                tid = srv.add_tenant(cfg["n"], src, cfg["m"], **kw)
            except T.TsvdError:
                continue  # not admitted: the HBM budget is spent
            srv.wait(srv.submit_update(tid, snaps[0]))
            tenants.append(dict(id=tid, n=int(n), rest=snaps[1], pos=0, cfg=cfg))
        t_setup = time.perf_counter() - t_setup
        stats0 = srv.stats()
        reqs = []
        t0 = time.perf_counter()
        next_t = t0
        with ClockSampler(device) as clk:
            for r in range(args.serve_requests):
                ten = tenants[int(rng.integers(len(tenants)))]
                hi = max(1e3, min(1e5, ten["cfg"]["m"] / 40))
                size = int(np.exp(rng.uniform(np.log(1e3), np.log(hi))))
                if ten["pos"] + size > len(ten["rest"]):
                    ten["pos"] = 0  # wrap: the batch re-inserts earlier pairs as duplicates
                e = ten["rest"][ten["pos"]:ten["pos"] + size]
                ten["pos"] += size
                next_t += rng.exponential(0.03)
                now = time.perf_counter()
                if next_t > now:
                    time.sleep(next_t - now)
                u = srv.submit_update(ten["id"], e)
                q = srv.submit_query(ten["id"])
                reqs.append((ten["n"], len(e), u, q))
            lat, svc = [], {}
            for n, m, u, q in reqs:
                l, sv, _ = srv.wait(u)
                srv.wait(q)
                lat.append(l)
                svc.setdefault(n, []).append(sv)
            wall = time.perf_counter() - t0
        edges = sum(m for _, m, _, _ in reqs)
        st = srv.stats()
    line = {"metric": "serving: p50/p99 refresh latency & edge updates/s, 1 GB300",
            "value": edges / wall, "unit": "edge updates/s", "n_gpus": 1,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "requests": len(reqs), "tenants_admitted": len(tenants),
            "tenants_offered": len(ns), "slots": args.serve_slots,
            "setup_s": t_setup, "stream_s": wall,
            "hbm_budget_gb": st["hbm_budget"] / 1e9, "hbm_charged_gb": st["hbm_charged"] / 1e9,
            "service_ms_mean_by_tenant_n": {str(n): float(np.mean(v)) for n, v in sorted(svc.items())},
            "clocks": clk.summary(), "higher_is_better": True,
            "data": "synthetic (seeded R-MAT tenants, Poisson arrivals)",
            "config": {"workload": "serve-%d-tenants" % len(ns), "tenant_n": [int(x) for x in ns],
                       "batch_edges": "log-uniform [1e3, min(1e5, M/40)]",
                       "arrivals": "Poisson, mean gap 30 ms", "alpha": 0.2, "rmax": 1e-7}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.serve:
        run_serve(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        tdist.barrier()
    cfg, snaps, sources = workload(args)
    res = run_ours(args, cfg, snaps, sources, local)
    if dist:
        import torch.distributed as tdist
        tdist.barrier()
    ms, edges_all, value = aggregate(res["ms"], res["edges"], f"cuda:{local}" if dist else None)
    lat = res["per_step"]
    line = {"metric": METRIC, "value": value, "unit": "edge updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 PPR state, f16 x (f16 hi+lo) tensor products, f32/f64 small solves",
            "data": "synthetic (seeded R-MAT, inputs resident in HBM; state >> L2)",
            "config": {"workload": cfg["name"], "n": cfg["n"], "m": cfg["m"],
                       "directed": cfg["directed"], "sources": cfg["sources"],
                       "n_parts": cfg["n_parts"], "rank_d": cfg["rank_d"],
                       "hierarchy_n": cfg["hierarchy_n"],
                       "passes_q": cfg["passes_q"], "snapshots": cfg["snapshots"],
                       "edges_per_step": res["edges"] / args.steps,
                       "l2": "working set (PPR state) larger than L2",
                       "parallelism": "replicas x%d" % world,
                       "ppr_reserve": "pinned host memory" if host_reserve(args, cfg) else "HBM",
                       "push_schedule": res["push_schedule"],
                       "driver": ("tsvd_session_run: factor stage of snapshot k overlapped "
                                  "with the push of k+1") if args.pipelined
                       else "tsvd_session_step per snapshot"},
            "setup_s": res["setup_s"],
            "clocks": res["clocks"], "gpu_launches": res["launches"],
            "stage_ms_mean": {k: float(np.mean([s[k] for s in res["stages"]]))
                              for k in ("ms_insert", "ms_refresh", "ms_push", "ms_log",
                                        "ms_frpca", "ms_merge")},
            "push_rounds_mean": float(np.mean([s["push_rounds"] for s in res["stages"]])),
            "pushes_mean": float(np.mean([s["pushes"] for s in res["stages"]])),
            "push_edge_updates_mean": float(np.mean([s["push_edge_updates"] for s in res["stages"]])),
            "push_items_mean": float(np.mean([s["push_items"] for s in res["stages"]])),
            "push_item_edges_mean": float(np.mean([s["push_item_edges"] for s in res["stages"]])),
            "ms_materialize_kernel_mean": float(np.mean([s["ms_materialize_kernel"] for s in res["stages"]])),
            "dirty_blocks_mean": float(np.mean([s["dirty_blocks"] for s in res["stages"]])),
            "sparse_blocks_mean": float(np.mean([s["sparse_blocks"] for s in res["stages"]])),
            "autotuner_density": float(res["stages"][-1]["tune_density"]),
            "eig_sweeps_merge_max": int(max(s["eig_sweeps_merge"] for s in res["stages"])),
            "merge_subspace_iters_max": int(max(s["merge_subspace_iters"] for s in res["stages"])),
            "eig_refine_sweeps_max": int(max(s["eig_refine_sweeps"] for s in res["stages"]))}
    line["roofline"] = push_roofline(res["stages"])
    line["tail"] = tail_attribution(res["stages"])
    if "e2e_ms" in res:
        line["e2e"] = {"value": res["e2e_edges"] * world / (res["e2e_ms"] / 1e3),
                       "unit": "edge updates/s", "steps": res["e2e_steps"],
                       "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                       "p50_ms": float(np.percentile(res["e2e_lat"], 50)),
                       "p99_ms": float(np.percentile(res["e2e_lat"], 99)),
                       "deltas": "the %d deltas after the timed ones, same session"
                                 % res["e2e_steps"]}
    if "plain" in res:
        pl = res["plain"]
        plat = pl["lat"]
        line["plain_form"] = {
            "form": "TSVD_FORM_PLAIN: one frontier entry and one scalar atomic per (vertex, "
                    "source) cell, fp64 push arithmetic on the fp32 state, FP32 CSR SpMM "
                    "frPCA one dirty block at a time, one merge per tree node",
            "steps": pl["steps"], "p50_ms": float(np.percentile(plat, 50)),
            "p99_ms": float(np.percentile(plat, 99)),
            "value": pl["edges"] / (pl["ms"] / 1e3), "unit": "edge updates/s",
            "stage_ms_mean": {k: float(np.mean([st[k] for st in pl["stages"]]))
                              for k in ("ms_insert", "ms_push", "ms_log", "ms_frpca",
                                        "ms_merge")},
            "deltas": "the %d deltas after the e2e leg, same session" % pl["steps"]}
        # the graph grows with every delta, so the plain leg (the last deltas)
        # is compared with the mixed form's latest snapshots: the e2e leg's
        # deltas when it ran (the ones just before), else the timed ones
        near = line.get("e2e", {}).get("p50_ms") or line["p50_ms"]
        line["p50_plain_over_mixed"] = line["plain_form"]["p50_ms"] / near
        line["p50_plain_over_mixed_basis"] = (
            "plain p50 / mixed e2e-leg p50 (adjacent deltas)" if line.get("e2e", {}).get("p50_ms")
            else "plain p50 / mixed timed p50")
    if rank == 0 and not args.no_cpu:
        info = cpu_sample(cfg, snaps, sources, steps=1,
                          k=args.cpu_sources or (os.cpu_count() or 1))
        s0 = info["steps"][0]
        line["cpu_baseline"] = {"value": s0["edges"] / s0["scaled_s"], "unit": "edge updates/s",
                                "cores": info["threads"], "kind": info["kind"],
                                "sample": info["sample"], "sample_wall_s": s0["wall_s"]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
