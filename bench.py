"""Benchmark: per-snapshot Tree-SVD refresh on one GB300 (or N replicas).

A step is one snapshot refresh of the named workload: insert the delta's
edges, refresh + push PPR (forward and reverse for directed graphs), log
transform + lazy test of every column block, frPCA of the dirty blocks, merge
of their ancestors. The first snapshot (half the edges, pushed from scratch)
is set-up and is not timed; the timed steps are later, dynamic snapshots.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "tree-embedding_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "p50/p99 re-embed latency & edge updates/s, 1 GB300, vs plain GPU form"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rmat-d-2.7m")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--sources", type=int, default=None)
    ap.add_argument("--parts", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--hierarchy", type=int, default=None,
                    help="merge arity (the workload's default is 2; the reference's run.sh uses 8)")
    ap.add_argument("--host-reserve", action="store_true",
                    help="keep the PPR reserve in pinned host memory (ppr_host_reserve), for "
                         "workloads whose state exceeds HBM (rmat-d-6.2m)")
    ap.add_argument("--pipelined", action="store_true",
                    help="time tsvd_session_run (factor stage of snapshot k overlapped with the "
                         "push of k+1: more snapshots/s, longer per-snapshot latency) instead of "
                         "one tsvd_session_step per snapshot")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--seed", type=int, default=20231)
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


def workload(args):
    import workloads as W
    cfg = W.scaled(args.workload, n=args.n, m=args.m, sources=args.sources, n_parts=args.parts)
    if args.hierarchy:
        cfg["hierarchy_n"] = args.hierarchy
    need = 1 + args.warmup + args.steps
    if cfg["snapshots"] < need:
        cfg["snapshots"] = need  # the second half of the edges is cut into more, smaller deltas
    edges, snaps, sources = W.build(cfg, seed=args.seed)
    return cfg, snaps, sources


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ------------------------------------------------------------------ our arm
def run_ours(args, cfg, snaps, sources, device):
    """Our arm. Each timed snapshot is one tsvd_session_step(_device) call, or
    with --pipelined all K go through one tsvd_session_run(_device) call (the
    factor stage of snapshot k overlapped with the push of snapshot k+1).
    Every snapshot is complete (embedding written) inside the timed region.
    Per-snapshot latency (stats ms_total) runs from the start of a snapshot's
    insert to the end of its factor stage."""
    import torch
    import tsvd_gb300 as T
    import workloads as W

    torch.cuda.set_device(device)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw["device"] = device
    kw["seed"] = args.seed
    kw["ppr_host_reserve"] = args.host_reserve
    t0i, t1i = 1 + args.warmup, 1 + args.warmup + args.steps
    timed = snaps[t0i:t1i]
    off = np.concatenate([[0], np.cumsum([len(e) for e in timed])]).astype(np.int64)
    # --- device-resident inputs: every delta uploaded before the timed region
    dev = [torch.from_numpy(np.ascontiguousarray(e)).to(f"cuda:{device}") for e in snaps[:t0i]]
    dev_timed = torch.from_numpy(np.ascontiguousarray(np.concatenate(timed))).to(f"cuda:{device}")
    res = {}
    with T.Session(cfg["n"], sources, **kw) as s:
        s.step_device(dev[0].data_ptr(), len(snaps[0]))  # set-up: first snapshot, from scratch
        for k in range(args.warmup):
            s.step_device(dev[1 + k].data_ptr(), len(snaps[1 + k]))
        stream = torch.cuda.ExternalStream(s.stream(), device=device)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = T.launch_count()
        torch.cuda.synchronize(device)
        with ClockSampler(device) as clk:
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
        launches = T.launch_count() - launches0
        ms = ev0.elapsed_time(ev1)
        res.update(ms=ms, wall=wall, per_step=[st["ms_total"] for st in stage], stages=stage,
                   launches=launches, clocks=clk.summary(), edges=int(off[-1]))
    del dev, dev_timed
    torch.cuda.empty_cache()
    if args.no_e2e:
        return res
    # --- end to end through the C-ABI: host edges (pinned) copied in and every
    # snapshot's embedding read back inside the timed region
    pinned_timed = torch.from_numpy(np.ascontiguousarray(np.concatenate(timed))).pin_memory()
    import ctypes
    with T.Session(cfg["n"], sources, **kw) as s:
        L = T.lib()
        for i in range(t0i):
            e = torch.from_numpy(np.ascontiguousarray(snaps[i])).pin_memory()
            T._check(L.tsvd_session_step(
                s._h, ctypes.cast(e.data_ptr(), ctypes.POINTER(ctypes.c_int32)), len(snaps[i])))
        emb = np.zeros((args.steps, len(sources), cfg["rank_d"]), np.float64)
        stats = (T.StepStats * args.steps)()
        stream = torch.cuda.ExternalStream(s.stream(), device=device)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        i32p, f64p = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
        ev0.record(stream)
        if args.pipelined:
            T._check(L.tsvd_session_run(
                s._h, ctypes.cast(pinned_timed.data_ptr(), i32p),
                off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), args.steps,
                emb.ctypes.data_as(f64p), stats))
        else:
            for k in range(args.steps):
                T._check(L.tsvd_session_step(
                    s._h, ctypes.cast(pinned_timed.data_ptr() + int(off[k]) * 8, i32p),
                    int(off[k + 1] - off[k])))
                T._check(L.tsvd_session_embedding(s._h, emb[k].ctypes.data_as(f64p)))
                T._check(L.tsvd_session_last_stats(s._h, ctypes.byref(stats[k])))
        ev1.record(stream)
        torch.cuda.synchronize(device)
        assert np.isfinite(emb).all()
        res["e2e_ms"] = ev0.elapsed_time(ev1)
        res["e2e_lat"] = [stats[k].ms_total for k in range(args.steps)]
        res["h2d"] = int(off[-1] * 8 / args.steps)
        res["d2h"] = int(len(sources) * cfg["rank_d"] * 4)
    return res


def cpu_sample(cfg, snaps, sources, budget_sources=None, threads=None):
    """Times the CPU oracle (the reference algorithm restated) on a bounded
    sample of one dynamic snapshot and scales it to the full workload:
    refresh + push on a subset of sources (cost is per source), one block's
    log transform + frPCA at full |S| (on a synthetic block of the measured
    density) and one merge, scaled by the blocks / merges of the snapshot."""
    from oracle import native
    from oracle.tree_oracle import frpca, log_transform
    import scipy.sparse as sp

    threads = threads or os.cpu_count() or 1
    S = len(sources)
    k = budget_sources or max(threads, min(S, 2 * threads))
    sub = np.sort(np.random.default_rng(0).choice(sources, k, replace=False)).astype(np.int32)
    n, alpha, rmax = cfg["n"], cfg["alpha"], cfg["rmax"]
    dirs = 2 if cfg["directed"] else 1
    g = native.OracleGraph(n, cfg["directed"])
    st = [native.OraclePPR(n, sub) for _ in range(dirs)]
    g.insert(snaps[0])
    for d in range(dirs):
        st[d].refresh(g, d, 1, 2, alpha, rmax, threads=threads)
        st[d].push(g, d, alpha, rmax, threads=threads)
    t = time.perf_counter()
    g.insert(snaps[1])
    for d in range(dirs):
        st[d].refresh(g, d, 2, 2, alpha, rmax, threads=threads)
        st[d].push(g, d, alpha, rmax, threads=threads)
    t_push = time.perf_counter() - t
    p = sum(x.reserve().astype(np.float64) for x in st)
    nparts = cfg["n_parts"]
    cd = n // nparts
    t = time.perf_counter()
    A = log_transform(p[:, :cd], rmax, cfg["transform"], n)
    t_log = (time.perf_counter() - t) * nparts
    density = np.count_nonzero(A) / A.size
    # one full-size block (|S| x n_b) of the measured density for frPCA
    rng = np.random.default_rng(1)
    nnz = int(density * S * cd)
    rows = rng.integers(0, S, nnz)
    cols = rng.integers(0, cd, nnz)
    vals = rng.uniform(0, np.log10(1 / rmax), nnz)
    B = sp.csr_matrix((vals, (rows, cols)), shape=(S, cd))
    omega = rng.standard_normal((cd, cfg["rank_d"] + 5))
    t = time.perf_counter()
    U, Sg, V = frpca(B, cfg["rank_d"], cfg["passes_q"], omega=omega)
    t_frpca = time.perf_counter() - t
    M = rng.standard_normal((S, cfg["hierarchy_n"] * cfg["rank_d"]))
    t = time.perf_counter()
    np.linalg.svd(M, full_matrices=False)
    t_merge = time.perf_counter() - t
    merges = nparts - 1
    est = t_push * S / k + t_log * S / k + t_frpca * nparts + t_merge * merges
    return {"seconds_per_snapshot": est, "edges": len(snaps[1]), "threads": threads,
            "sample": ("one dynamic snapshot (%d edges): refresh+push on %d of %d sources "
                       "(%.2fs, scaled x%.1f), log transform of one block (x%d), frPCA of one "
                       "%dx%d block at density %.3f (%.2fs, x%d blocks), one %dx%d merge SVD "
                       "(x%d); all blocks assumed dirty" % (
                           len(snaps[1]), k, S, t_push, S / k, nparts, S, cd, density, t_frpca,
                           nparts, S, cfg["hierarchy_n"] * cfg["rank_d"], merges))}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cfg, snaps, sources = workload(args)
    vals = []
    info = None
    t0 = time.perf_counter()
    # each step is one bounded CPU sample of a dynamic snapshot, scaled to the
    # full workload; the run stops after two minutes of samples
    for k in range(max(1, args.steps)):
        info = cpu_sample(cfg, snaps, sources)
        vals.append(info["edges"] / info["seconds_per_snapshot"])
        if time.perf_counter() - t0 > 120:
            break
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "edge updates/s",
            "n_gpus": args.gpus, "steps": len(vals), "warmup": args.warmup,
            "ms_per_step": info["edges"] / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 state / f64 arithmetic",
            "data": "synthetic (seeded R-MAT)",
            "config": {"workload": args.workload, "n": cfg["n"], "m": cfg["m"],
                       "sources": cfg["sources"], "n_parts": cfg["n_parts"]},
            "cpu_baseline": {"value": v, "unit": "edge updates/s", "cores": info["threads"],
                             "kind": "port", "sample": info["sample"]},
            "e2e": {"value": v, "unit": "edge updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# DRAM bytes (read + write) of push_kernel + push_heavy_kernel per pushed
# item-neighbour (one 256-byte residue-run atomic), from one ncu capture of
# every push launch of a timed rmat-d-2.7m snapshot (dram__bytes_read.sum +
# dram__bytes_write.sum, one pass): 2443.6 GB over 7.615e9 item-neighbours,
# one 256-byte run atomic each (profiles/push_kernel_rmat-d-2.7m.md).
# `traffic` scales it to the launches of the run being reported.
PUSH_TRAFFIC_BYTES_PER_ITEM_EDGE = 320.9


def push_roofline(stages):
    """Roofline of the dominant kernels (push_kernel + push_heavy_kernel) over
    the timed steps, duration from CUDA events around every launch on the
    session stream.

    Algorithmic bytes (`achieved`) follow the per-push work of the reference's
    FIFO push: per executed push of (v, s) 8 (r_v read) + 8 (r_v write) + 16
    (p_v read-modify-write) + 8 (row offsets), and per edge update 4
    (neighbour id) + 16 (r_u atomic read-modify-write).

    `achieved_min` counts the bytes this design has to move at least: per lane
    push 16 (fp32 residue exchange + reserve update), per lane edge update 8
    (fp32 atomic read-modify-write), per item-neighbour 4 (the neighbour id is
    read once for the 64 sources of a chunk), per item 20 (frontier entry, row start,
    degree)."""
    pk, _ = peaks()
    peak = float(pk.get("hbm_gbs", 6800.0))
    pushes = sum(s["pushes"] for s in stages)
    upd = sum(s["push_edge_updates"] for s in stages)
    items = sum(s["push_items"] for s in stages)
    iedges = sum(s["push_item_edges"] for s in stages)
    ms = sum(s["ms_push_kernels"] for s in stages)
    launches = sum(2 * s["push_rounds"] for s in stages)
    byts = 40.0 * pushes + 20.0 * upd
    byts_min = 16.0 * pushes + 8.0 * upd + 4.0 * iedges + 20.0 * items
    sec = ms / 1e3
    achieved = byts / sec / 1e9 if ms > 0 else 0.0
    achieved_min = byts_min / sec / 1e9 if ms > 0 else 0.0
    traffic = None
    if PUSH_TRAFFIC_BYTES_PER_ITEM_EDGE is not None and launches:
        traffic = PUSH_TRAFFIC_BYTES_PER_ITEM_EDGE * iedges / launches
    return {"kernel": "push_kernel+push_heavy_kernel", "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "algorithmic_bytes_per_launch": byts / max(1, launches),
            "achieved_min": achieved_min, "frac_min": achieved_min / peak,
            "min_bytes_per_launch": byts_min / max(1, launches),
            "launches": launches, "kernel_ms": ms,
            "lanes_per_item": pushes / max(1, items),
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth), of measured"}


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


def main():
    args = parse()
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
            "config": {"workload": args.workload, "n": cfg["n"], "m": cfg["m"],
                       "directed": cfg["directed"], "sources": cfg["sources"],
                       "n_parts": cfg["n_parts"], "rank_d": cfg["rank_d"],
                       "hierarchy_n": cfg["hierarchy_n"],
                       "passes_q": cfg["passes_q"], "snapshots": cfg["snapshots"],
                       "l2": "working set (PPR state) larger than L2",
                       "parallelism": "replicas x%d" % world,
                       "ppr_reserve": "pinned host memory" if args.host_reserve else "HBM",
                       "driver": ("tsvd_session_run: factor stage of snapshot k overlapped "
                                  "with the push of k+1") if args.pipelined
                       else "tsvd_session_step per snapshot"},
            "clocks": res["clocks"], "gpu_launches": res["launches"],
            "stage_ms_mean": {k: float(np.mean([s[k] for s in res["stages"]]))
                              for k in ("ms_insert", "ms_push", "ms_log", "ms_frpca", "ms_merge")},
            "push_rounds_mean": float(np.mean([s["push_rounds"] for s in res["stages"]])),
            "pushes_mean": float(np.mean([s["pushes"] for s in res["stages"]])),
            "push_edge_updates_mean": float(np.mean([s["push_edge_updates"] for s in res["stages"]])),
            "push_items_mean": float(np.mean([s["push_items"] for s in res["stages"]])),
            "push_item_edges_mean": float(np.mean([s["push_item_edges"] for s in res["stages"]])),
            "ms_materialize_kernel_mean": float(np.mean([s["ms_materialize_kernel"] for s in res["stages"]])),
            "dirty_blocks_mean": float(np.mean([s["dirty_blocks"] for s in res["stages"]])),
            "eig_sweeps_merge_max": int(max(s["eig_sweeps_merge"] for s in res["stages"])),
            "merge_subspace_iters_max": int(max(s["merge_subspace_iters"] for s in res["stages"])),
            "eig_refine_sweeps_max": int(max(s["eig_refine_sweeps"] for s in res["stages"]))}
    line["roofline"] = push_roofline(res["stages"])
    if "e2e_ms" in res:
        line["e2e"] = {"value": edges_all / (res["e2e_ms"] / 1e3), "unit": "edge updates/s",
                       "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                       "p50_ms": float(np.percentile(res["e2e_lat"], 50)),
                       "p99_ms": float(np.percentile(res["e2e_lat"], 99))}
    if rank == 0 and not args.no_cpu:
        info = cpu_sample(cfg, snaps, sources)
        cv = info["edges"] / info["seconds_per_snapshot"]
        line["cpu_baseline"] = {"value": cv, "unit": "edge updates/s", "cores": info["threads"],
                                "kind": "port", "sample": info["sample"]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
