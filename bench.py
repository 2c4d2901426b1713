#!/usr/bin/env python
"""Benchmark of the refine sweep (the headline of this repository).

Workload (N=1): R-MAT scale 24, edge factor 16, quadrants (.57, .19, .19, .05),
seed 2, random vertex permutation, loops/duplicates/isolated vertices removed
and vertices renumbered by decreasing degree as the reference converter does.
One step = one synchronous label-propagation sweep with the Modularity rule,
frac 1.0; the timed steps cycle through the first five sweeps of the
reference's -s 0 schedule, each restored from a device copy of its start
partition and run with that sweep's rand_r seed (compress + statistics of
the start partition are done before the timed sweep).

Lines printed (rank 0, one JSON line):
  value      refine-sweep edges/s, inputs resident in HBM, CUDA events on the
             stream the kernels run on, max over ranks
  e2e        the same metric through the C ABI with HOST buffers: every step
             loads the CSR from pinned host memory, sets the start labels,
             sweeps, and reads the labels back (the same cycle of sweeps)
  roofline   the sweep's dominant kernel against the measured HBM copy peak
  cpu_baseline  the oracle (C restatement of the reference, OpenMP) on the
             host cores, on the same graph
  batched    4096 log-normal SBMs through pcd_batch_run vs the single-graph
             path looped over a sample vs the oracle driver loop on the CPU
  served     Poisson arrivals (SBM / power-law / R-MAT s22 mix) through the
             serving loop vs the single-graph path one request at a time:
             graphs/s and latency percentiles
  convert    the workload's raw edge list through the GPU converter
  extras     connected components and NMI on the workload graph, the
             triangle-based initial partition on R-MAT scale 22
With --impl reference: the reference's CPU path for this sweep (the oracle
restatement; the reference's own objects cannot run on this host) on all host
cores, same metric and workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "par-cd_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "refine-sweep edges/s (% of HBM roofline); batched graphs/s + p99 vs plain"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def tune_cache() -> str:
    import tempfile

    return os.path.join(tempfile.gettempdir(), "pcd_bench_tuning.json")


def max_over_ranks(dist, x: float, device) -> float:
    """The job's time is its slowest rank's: max of x over the ranks (x itself
    without a process group)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(args, device):
    import graphs

    t0 = time.time()
    if args.scale >= 16:
        ind, adj, _ = graphs.rmat_torch(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=2, device=device)
    else:
        g = graphs.convert_edges(graphs.rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=2))
        ind, adj = g.indices, g.adj
    log(f"[bench] R-MAT s{args.scale}: n={ind.shape[0] - 1} m={adj.shape[0] // 2} ({time.time() - t0:.1f}s)")
    return ind, adj


def bins_bytes(ind, bounds=(4, 8, 16, 32, 256, 2048, 8192)):
    """Algorithmic bytes per vertex class: 8 deg + 12 (row offsets, adjacency,
    neighbour-label gathers, own label read, new label write); `bounds` are
    the classes' upper degrees (the graph's degree classes)."""
    import numpy as np

    deg = np.diff(ind.astype(np.int64))
    edges = [0] + [int(x) for x in bounds] + [1 << 62]
    names = ["sweep.g4", "sweep.g8", "sweep.g16", "sweep.g32", "sweep.warp", "sweep.block", "sweep.block_l",
             "sweep.hub"]
    out = {}
    for nm, lo, hi in zip(names, edges[:-1], edges[1:]):
        sel = (deg > lo) & (deg <= hi) if lo else (deg <= hi)
        out[nm] = int(8 * deg[sel].sum() + 12 * sel.sum())
    return out


def cpu_sweeps(ind, adj, seeds, threads, steps, budget_s):
    """The oracle's OpenMP propagation sweeps (Modularity, frac 1.0) on the
    host cores: the schedule's first len(seeds) sweeps from the singleton
    partition (each sweep starts from the compressed result of the previous
    one), cycled for `steps` sweeps or until `budget_s` seconds are spent.
    Returns (edges/s, sweeps timed, seconds)."""
    import numpy as np

    import oracle

    port = oracle.Port()
    port.load(ind, adj)
    n = ind.shape[0] - 1
    m = adj.shape[0] // 2
    lab = np.arange(n, dtype=np.int32)
    starts = []
    times = []
    t_all = time.time()
    for i in range(steps):
        j = i % len(seeds)
        if j < len(starts):
            lab = starts[j]
        else:
            lab, _ = port.compress(lab)
            starts.append(lab)
        st = port.stats(lab)
        t0 = time.perf_counter()
        out = port.refine_prop(0, 0.0, lab, 1.0, seed=seeds[j], threads=threads, st=st)
        times.append(time.perf_counter() - t0)
        lab = out
        if time.time() - t_all > budget_s:
            break
    sec = sum(times)
    return m * len(times) / sec, len(times), sec


def schedule_seeds(ind, adj, count):
    """The rand_r seeds of the schedule's first `count` refinement calls: the
    reference's glibc rand() stream (seed 1) after create_singleton_partition's
    n draws.  Drawn through the oracle's restatement of rand(), so the
    reference arm maps no library of the product."""
    import oracle

    port = oracle.Port()
    port.load(ind, adj)
    port.singleton()
    return [port.rand() for _ in range(count)]


def oracle_sweep_parity(ind, adj, starts, seeds, gpu_out, budget_s):
    """Bit-exact check of the timed sweeps: the oracle's single-threaded
    PropagationRefinement::refine (the reference's -p 1 schedule) from each
    sweep's start partition with its seed, against the GPU's labels of the
    same sweep.  The sweeps run side by side on host threads (the oracle's C
    call releases the interpreter lock).  Returns a dict for the JSON line."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor

    import oracle

    port = oracle.Port()
    port.load(ind, adj)
    t0 = time.time()

    def one(j):
        st = port.stats(starts[j])
        want = port.refine_prop(0, 0.0, starts[j], 1.0, seed=seeds[j], threads=1, st=st)
        return j, int(np.count_nonzero(want != gpu_out[j]))

    with ThreadPoolExecutor(max(1, min(len(starts), os.cpu_count() or 1))) as ex:
        res = list(ex.map(one, range(len(starts))))
    diff = {j: d for j, d in res}
    return {"sweeps_checked": len(res), "bit_exact": all(d == 0 for d in diff.values()),
            "labels_differing": [diff[j] for j in range(len(res))],
            "oracle": "single-threaded C restatement of PropagationRefinement::refine (-p 1 schedule)",
            "seconds": round(time.time() - t0, 1)}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    import torch

    dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    ind, adj = make_workload(args, dev)
    n = ind.shape[0] - 1
    m = adj.shape[0] // 2
    seeds = schedule_seeds(ind, adj, args.sweeps)
    threads = os.cpu_count() or 1
    if args.warmup:
        cpu_sweeps(ind, adj, seeds[:1], threads, 1, 60.0)
    value, k, sec = cpu_sweeps(ind, adj, seeds, threads, max(1, args.steps), 180.0)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "edges/s",
        "n_gpus": world,
        "steps": k,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * sec / k,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32 labels, fp64 gains",
        "data": "synthetic",
        "config": workload_config(args, n, m),
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{k} propagation sweeps (the schedule's first {args.sweeps}, cycled) of the "
                                   f"workload graph by the oracle's OpenMP restatement of "
                                   f"PropagationRefinement::refine on {threads} host threads (-p {threads}), "
                                   f"{sec:.1f}s; the restatement is pinned bit-exact to the reference's own "
                                   f"objects at -p 1 (the reference's objects are not built on this host)"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def batch_cpu_baseline(voff, ind, adj, idx, sched, budget_s):
    """The oracle's driver loop (one host thread per graph, all host cores in
    parallel) over the sampled graphs until `budget_s` is spent: graphs/s."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np

    import oracle

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    done = []

    def one(i):
        if time.perf_counter() - t0 > budget_s:
            return None
        a, b = int(voff[i]), int(voff[i + 1])
        li = (ind[a:b + 1] - ind[a]).astype(np.int32)
        la = adj[int(ind[a]):int(ind[b])]
        oracle.run_schedule(oracle.Port(), li, la, sched["metric"], sched["strategy"], sched["frac"],
                            sched["rounds"], sched["n_iter"], sched["threshold"], 0, 1)
        return i

    with ThreadPoolExecutor(threads) as ex:
        for r in ex.map(one, idx):
            if r is not None:
                done.append(r)
    sec = time.perf_counter() - t0
    return len(done) / sec, len(done), sec, threads


def batched_leg(args, ctx, dev, strategy=None, frac=None):
    """Many-graph workload: the log-normal batch of SBMs, every graph run
    through the reference driver's schedule (singleton start, stop test,
    final labels and score).  Batched = one packed batch through
    pcd_batch_run (CUDA-graph-captured iterations); plain = the same graphs
    one after another through the single-graph API.  Both arms start from the
    graphs' CSR resident in HBM and end with every label and score on the
    host; per-graph labels, scores and iteration counts must be identical."""
    import numpy as np
    import torch

    import graphs
    import pcd

    t0 = time.time()
    voff, d_ind, d_adj = graphs.sbm_batch_torch(args.batch_graphs, seed=4, device=dev)
    torch.cuda.synchronize()
    Gn = voff.shape[0] - 1
    N = int(voff[-1])
    M = int(d_ind[-1].item()) // 2
    log(f"[bench] batch: {Gn} SBM graphs, n={N} m={M} ({time.time() - t0:.1f}s)")
    sched = {"metric": args.batch_metric,
             "strategy": args.batch_strategy if strategy is None else strategy,
             "frac": args.batch_frac if frac is None else frac,
             "rounds": 1, "n_iter": args.batch_iters, "threshold": args.batch_threshold}
    rule = pcd.parse_metric(sched["metric"])
    h_labels = torch.empty(N, dtype=torch.int32).pin_memory()
    tuned = None
    if args.tune:
        import tune

        Bt = pcd.Batch.from_device(ctx, voff, d_ind.data_ptr(), d_adj.data_ptr())
        tr = tune.tune_batch(Bt, rule, sched["frac"], d_ind.cpu().numpy(), cache_path=tune_cache(), retune=True)
        Bt.free()
        tuned = {k: tr[k] for k in ("bins", "hub_part", "ms", "default_ms")}
        tuned["note"] = "ms: the batch's first propagation step, best tuned vs default classes"

    def configure(B):
        if tuned:
            B.set_bins(tuned["bins"])
            B.set_hub_part(tuned["hub_part"])

    def batched_job():
        B = pcd.Batch.from_device(ctx, voff, d_ind.data_ptr(), d_adj.data_ptr())
        configure(B)
        scores, iters = B.run(rule, sched["strategy"], sched["frac"], sched["rounds"], sched["n_iter"],
                              sched["threshold"], True)
        B.get_labels_ptr(h_labels.data_ptr())
        B.free()
        return scores, iters

    scores, iters = batched_job()  # warm-up (and the results checked below)
    labels_b = h_labels.numpy().copy()
    times = []
    for _ in range(max(1, args.batch_reps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        s2, i2 = batched_job()
        times.append(time.perf_counter() - t)
        assert np.array_equal(s2, scores) and np.array_equal(i2, iters), "batched run not repeatable"
    batched_s = statistics.median(times)

    # end to end from pinned host buffers
    h_ind = d_ind.cpu().pin_memory()
    h_adj = d_adj.cpu().pin_memory()
    torch.cuda.synchronize()
    t = time.perf_counter()
    B = pcd.Batch.from_host_ptr(ctx, voff, h_ind.data_ptr(), h_adj.data_ptr())
    configure(B)
    s3, _ = B.run(rule, sched["strategy"], sched["frac"], sched["rounds"], sched["n_iter"], sched["threshold"],
                  True)
    B.get_labels_ptr(h_labels.data_ptr())
    B.free()
    e2e_s = time.perf_counter() - t
    assert np.array_equal(s3, scores)

    # the plain path, looped over a stride sample of the same graphs
    stride = max(1, args.batch_plain_stride)
    idx = list(range(0, Gn, stride))
    ind_h = h_ind.numpy()
    loc = []
    for i in idx:
        a, b = int(voff[i]), int(voff[i + 1])
        li = (d_ind[a:b + 1] - d_ind[a]).contiguous()
        loc.append((i, li, d_adj[int(ind_h[a]):].data_ptr(), b - a, int(ind_h[b] - ind_h[a]) // 2))
    torch.cuda.synchronize()
    mism = 0
    t = time.perf_counter()
    for i, li, adj_ptr, n_g, m_g in loc:
        g1 = pcd.Graph.from_device(ctx, n_g, m_g, li.data_ptr(), adj_ptr)
        res = pcd.run(g1, rule, sched["strategy"], sched["frac"], sched["rounds"], sched["n_iter"],
                      sched["threshold"], 0)
        g1.free()
        if not (res.score == scores[i] and res.iterations == iters[i]
                and np.array_equal(res.labels, labels_b[voff[i]:voff[i + 1]])):
            mism += 1
    plain_s = time.perf_counter() - t
    assert mism == 0, f"{mism} graphs differ between the batched and the plain path"
    plain_gps = len(idx) / plain_s
    batched_gps = Gn / batched_s
    sample_edges = sum(x[4] for x in loc)

    cpu = None
    if not args.no_cpu:
        adj_h = h_adj.numpy()
        v, k, sec, thr = batch_cpu_baseline(voff, ind_h, adj_h, idx, sched, 20.0)
        cpu = {"value": v, "unit": "graphs/s", "cores": thr, "kind": "port",
               "sample": f"{k} graphs of the stride-{stride} sample, oracle driver loop, one graph per host "
                         f"thread, {thr} threads, {sec:.1f}s"}
    return {
        "workload": f"{Gn} SBM graphs, n ~ LogNormal(ln 5000, 1.2) clipped to [200, 300000], n/50 blocks, "
                    f"intra-degree 12, inter-degree 2, seed 4 (device generator), degree-sorted",
        "schedule": f"-m {sched['metric']} -s {sched['strategy']} -f {sched['frac']} -n {sched['n_iter']} "
                    f"-t {sched['threshold']} from singletons",
        "n": N, "m": M,
        "graphs_per_s": batched_gps,
        "ms_per_job": 1000.0 * batched_s,
        "edges_per_s": M / batched_s,
        "e2e": {"graphs_per_s": Gn / e2e_s, "ms_per_job": 1000.0 * e2e_s,
                "h2d_bytes": int(4 * (N + 1) + 8 * M + 4 * (Gn + 1)), "d2h_bytes": int(4 * N + 12 * Gn)},
        "plain_graphs_per_s": plain_gps,
        "plain_sample": f"every {stride}th graph ({len(idx)} graphs, m={sample_edges}), {plain_s:.2f}s",
        "speedup_vs_plain": batched_gps / plain_gps,
        "iterations_max": int(iters.max()), "iterations_mean": float(iters.mean()),
        "identical_to_plain": True,
        "tuning": tuned,
        "cpu_baseline": cpu,
    }


def convert_leg(args, dev, ind, adj):
    """The converter on the GPU: the workload's raw R-MAT edge list (loops and
    duplicates included) from host memory through pcd_convert_edges, timed
    end to end (H2D copy, sorts, CSR, load as a graph); its CSR must equal the
    workload's.  CPU: the host restatement of the reference converter on the
    scale-20 edge list of the same generator."""
    import numpy as np
    import torch

    import graphs
    import pcd

    src, dst = graphs.rmat_edges_torch(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=2, device=dev)
    e = torch.stack([src, dst], 1).to(torch.int32).cpu().numpy()
    del src, dst
    torch.cuda.empty_cache()
    ctx = pcd.Context(0)
    g, _ = pcd.convert_edges(ctx, e[:1000])  # warm-up
    g.free()
    torch.cuda.synchronize()
    t = time.perf_counter()
    g, mp = pcd.convert_edges(ctx, e)
    sec = time.perf_counter() - t
    gi, ga = g.csr()
    same = bool(np.array_equal(gi, ind) and np.array_equal(ga, adj))
    g.free()
    ctx.close()
    out = {"edges_in": int(e.shape[0]), "n": int(gi.shape[0] - 1), "m": int(ga.shape[0] // 2),
           "seconds": sec, "input_edges_per_s": e.shape[0] / sec, "same_csr_as_workload": same}
    if not args.no_cpu:
        src, dst = graphs.rmat_edges_torch(20, args.edge_factor, 0.57, 0.19, 0.19, seed=2, device=dev)
        e20 = torch.stack([src, dst], 1).cpu().numpy()
        t = time.perf_counter()
        graphs.convert_edges(e20, 1 << 20)
        c = time.perf_counter() - t
        out["cpu_baseline"] = {"value": e20.shape[0] / c, "unit": "input edges/s", "cores": 1, "kind": "port",
                               "sample": f"R-MAT s20 edge list ({e20.shape[0]} edges), numpy restatement of the "
                                         f"reference converter, {c:.1f}s"}
    assert same, "the GPU converter's CSR differs from the workload's"
    log(f"[bench] convert: {e.shape[0]} edges in {sec:.2f}s")
    return out


def extras_leg(args, dev, ind, adj):
    """The rows beside the sweep, on the GPU: FindConnectedRefinement
    (pcd_find_connected) on the workload graph, the NMI (pcd_nmi_device) of
    two synthetic labelings of its vertices; the triangle-based
    initial partition (pcd_clustering_partition_device, triangles counted
    first and timed apart) on the R-MAT scale-22 graph of the same generator.
    Wall time of each call (each synchronises), after one warm-up call.  CPU:
    the oracle's restatements of the same functions on the scale-18 graph."""
    import numpy as np
    import torch

    import graphs
    import pcd

    def timed(f):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = f()
        return r, time.perf_counter() - t

    ctx = pcd.Context(0)
    out = {}
    G = pcd.Graph.from_csr(ctx, ind, adj)
    fc = pcd.FindConnectedRefinement()
    fc.refine(G)
    k, sec = timed(lambda: fc.refine(G))
    n = G.n
    out["find_connected"] = {"graph": f"rmat-s{args.scale}", "components": k, "ms": 1000 * sec,
                             "edges_per_s": G.m / sec}
    # two synthetic labelings of the workload's vertices (the components'
    # giant part would overflow the reference's int product ni * nj)
    vid = torch.arange(n, device=dev, dtype=torch.int64)
    la = ((vid * 7919) % 9973).to(torch.int32)
    lb = (vid // 997).to(torch.int32)
    pcd.nmi(ctx, la, lb, n)
    v, sec = timed(lambda: pcd.nmi(ctx, la, lb, n))
    out["nmi"] = {"graph": f"rmat-s{args.scale}", "pairs": n, "value": v, "ms": 1000 * sec,
                  "pairs_per_s": n / sec}
    G.free()
    del vid, la, lb
    i22, a22, _ = graphs.rmat_torch(22, args.edge_factor, 0.57, 0.19, 0.19, seed=2, device=dev)
    torch.cuda.empty_cache()
    G = pcd.Graph.from_csr(ctx, i22, a22)
    _, tsec = timed(lambda: G.count_triangles())
    pcd.create_clustering_partition_device(G)
    k, sec = timed(lambda: pcd.create_clustering_partition_device(G))
    out["clustering_partition"] = {"graph": "rmat-s22", "n": G.n, "m": G.m, "communities": k,
                                   "ms": 1000 * sec, "triangles_ms": 1000 * tsec, "vertices_per_s": G.n / sec}
    G.free()
    ctx.close()
    if not args.no_cpu:
        import oracle

        i18, a18, _ = graphs.rmat_torch(18, args.edge_factor, 0.57, 0.19, 0.19, seed=2, device=dev)
        port = oracle.Port().load(i18, a18)
        port.count_triangles()
        t = time.perf_counter()
        port.clustering()
        c1 = time.perf_counter() - t
        t = time.perf_counter()
        port.find_connected()
        c2 = time.perf_counter() - t
        n18 = i18.shape[0] - 1
        vid = np.arange(n18, dtype=np.int64)
        t = time.perf_counter()
        port.nmi(((vid * 7919) % 9973).astype(np.int32), (vid // 997).astype(np.int32))
        c3 = time.perf_counter() - t
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": f"R-MAT s18 (n {n18}, m {a18.shape[0] // 2})",
                               "clustering_partition_vertices_per_s": n18 / c1,
                               "find_connected_edges_per_s": (a18.shape[0] // 2) / c2,
                               "nmi_pairs_per_s": n18 / c3}
    log(f"[bench] extras: {json.dumps(out)}")
    return out


def serve_pool(dev):
    """The served mix's graphs (seed 5): SBMs with log-uniform sizes in
    [1000, 50000] (n/50 blocks, intra-degree 12, inter-degree 2), LFR-style
    power-law graphs (degree exponent 2.5 in [8, 5000], community sizes 1.5 in
    [20, 20000], mu 0.3) and one R-MAT scale 22; host CSR arrays."""
    import numpy as np
    import torch

    import graphs

    rng = np.random.default_rng(5)
    ns = np.rint(np.exp(rng.uniform(np.log(1000), np.log(50000), 64))).astype(np.int64)
    voff, ind, adj = graphs.sbm_batch_torch(len(ns), seed=5, device=dev, sizes=ns)
    sbm = graphs.unpack(voff, ind.cpu().numpy(), adj.cpu().numpy())
    pl = []
    for k, n in enumerate((100_000, 250_000, 600_000)):
        e = graphs.powerlaw(n, 2.5, 8, 5000, 1.5, 20, 20000, 0.3, seed=50 + k)
        i, a, _ = graphs.csr_from_edges_torch(torch.from_numpy(e[:, 0]).to(dev), torch.from_numpy(e[:, 1]).to(dev), n)
        pl.append((i, a))
    i, a, _ = graphs.rmat_torch(22, 16, 0.57, 0.19, 0.19, seed=5, device=dev)
    torch.cuda.empty_cache()
    return sbm, pl, [(i, a)]


def served_leg(args, dev):
    """Requests arrive as a Poisson stream (seed 5): 90% SBM, 9% power-law, 1%
    R-MAT s22, each Modularity or CPM(0.01), -s 0 -f 1.0 with the iteration
    count pinned (-n, default 20: under CPM an R-MAT graph's score never turns
    positive, so a -t 0 stop test would run it to the iteration cap).
    Served: pcd.Server with continuous batching (graphs join and leave running
    batches between iterations, under a 150 GB HBM budget).  Plain: the same
    requests in arrival order through the single-graph path, one at a time
    (FIFO queue: latency = wait + service).  Arrival rates are multiples of the
    plain path's capacity (1 / mean service time), from well below it to well
    above it.  Every served result must equal the plain one."""
    import numpy as np

    import pcd

    t0 = time.time()
    sbm, pl, rm = serve_pool(dev)
    log(f"[bench] serve pool: {len(sbm)} SBM, {len(pl)} power-law, {len(rm)} R-MAT s22 ({time.time() - t0:.1f}s)")
    rng = np.random.default_rng(5)
    reqs, kinds = [], []
    for _ in range(args.serve_requests):
        u = rng.random()
        pool = sbm if u < 0.90 else (pl if u < 0.99 else rm)
        g = pool[int(rng.integers(len(pool)))]
        reqs.append((g, "mod" if rng.random() < 0.5 else "cpm-0.01"))
        kinds.append("sbm" if u < 0.90 else ("powerlaw" if u < 0.99 else "rmat22"))
    n_iter = args.serve_iters
    gaps = rng.exponential(1.0, size=len(reqs))
    edges = sum(len(g[1]) // 2 for g, _ in reqs)

    # plain: service times, one request after another
    ctx = pcd.Context(int(str(dev).split(":")[-1]) if ":" in str(dev) else 0)
    plain = []
    for g, metric in reqs[:3]:  # warm-up
        G = pcd.Graph.from_csr(ctx, g[0], g[1])
        pcd.run(G, pcd.parse_metric(metric), 0, 1.0, 1, n_iter, 0.0, 0)
        G.free()
    for g, metric in reqs:
        t = time.perf_counter()
        G = pcd.Graph.from_csr(ctx, g[0], g[1])
        res = pcd.run(G, pcd.parse_metric(metric), 0, 1.0, 1, n_iter, 0.0, 0)
        G.free()
        plain.append((time.perf_counter() - t, res))
    ctx.close()
    service = np.array([p[0] for p in plain])

    def pct(x):
        return {k: round(float(np.percentile(x, q)) * 1000.0, 3) for k, q in (("p50", 50), ("p90", 90), ("p99", 99))} | \
               {"max": round(float(np.max(x)) * 1000.0, 3)}

    plain_capacity = 1.0 / float(np.mean(service))
    rates = [m * plain_capacity for m in args.serve_rate_multiples] if not args.serve_rates else args.serve_rates
    out = {"requests": len(reqs), "edges": int(edges),
           "mix": "90% SBM n~LogUniform[1e3, 5e4] (64-graph pool), 9% power-law n in {1e5, 2.5e5, 6e5}, "
                  f"1% R-MAT s22; mod or cpm-0.01 each with p 1/2; -s 0 -f 1.0 -n {n_iter} from singletons",
           "plain_capacity_graphs_per_s": plain_capacity,
           "hbm_budget_bytes": 150 * 10**9, "rates": [],
           "plain_service_by_type": {k: {"requests": int(sum(1 for x in kinds if x == k)),
                                         "mean_ms": round(1000.0 * float(np.mean([service[i] for i in range(len(reqs))
                                                                                  if kinds[i] == k])), 3),
                                         "mean_iterations": float(np.mean([plain[i][1].iterations
                                                                           for i in range(len(reqs))
                                                                           if kinds[i] == k]))}
                                     for k in ("sbm", "powerlaw", "rmat22") if k in kinds}}
    for rate in rates:
        # each rate serves the first `cnt` requests: about serve_seconds of arrivals
        cnt = int(min(len(reqs), max(100, rate * args.serve_seconds)))
        sub = reqs[:cnt]
        arrival = np.cumsum(gaps[:cnt] / rate)
        # plain FIFO queue
        fin = np.zeros(cnt)
        prev = 0.0
        for k in range(cnt):
            prev = max(arrival[k], prev) + service[k]
            fin[k] = prev
        plain_lat = fin - arrival
        with pcd.Server(device=0, workers=args.serve_workers, max_batch_graphs=256,
                        hbm_budget_bytes=150 * 10**9, max_wait_ms=2.0, continuous=True) as srv:
            tickets = []
            start = time.perf_counter()
            for k, (g, metric) in enumerate(sub):
                delay = start + arrival[k] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(g[0], g[1], pcd.parse_metric(metric), 0, 1.0, 1, n_iter, 0.0))
            lat, same = [], 0
            for k, t in enumerate(tickets):
                r = srv.wait(t)
                lat.append(r.latency_ms / 1000.0)
                p = plain[k][1]
                same += int(np.array_equal(r.labels, p.labels) and r.score == p.score and r.iterations == p.iterations)
            wall = time.perf_counter() - start
            st = srv.stats()
        assert same == cnt, f"{cnt - same} served results differ from the plain path"
        lat = np.array(lat)
        out["rates"].append({
            "arrival_rate": rate,
            "rate_vs_plain_capacity": rate / plain_capacity,
            "requests": cnt,
            "served": {"graphs_per_s": cnt / wall, "latency_ms": pct(lat), "batches": st["batches"],
                       "mean_batch_graphs": st["batched_graphs"] / max(1, st["batches"]),
                       "admitted_into_running_batches": st["admitted_running"],
                       "returned_while_batch_ran_on": st["released_early"],
                       "hbm_peak_estimated_bytes": st["bytes_peak"], "hbm_batch_measured_peak_bytes":
                           st["bytes_measured_peak"], "estimate_exceeded": st["estimate_exceeded"]},
            "plain": {"graphs_per_s": cnt / float(fin[-1]), "latency_ms": pct(plain_lat)},
            "identical_to_plain": True,
        })
        log(f"[bench] served at {rate}/s: {out['rates'][-1]['served']['graphs_per_s']:.0f} graphs/s, "
            f"p99 {out['rates'][-1]['served']['latency_ms']['p99']} ms (plain p99 "
            f"{out['rates'][-1]['plain']['latency_ms']['p99']} ms)")
    return out


def timed_sweeps(G, rule, start, seed, reps, stream):
    """CUDA-event times (ms) of `reps` propagation sweeps (frac 1.0), each
    from the device labels `start` with rand_r seed `seed`; the compress and
    statistics of the start partition run before each timed sweep."""
    import torch

    import pcd

    sweep = pcd.PropagationRefinement(1.0)
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            G.set_labels_device(start.data_ptr())
            G.compress(sync=False)
            e0.record(stream)
            sweep.refine(G, rule, seed)
            e1.record(stream)
        stream.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms


def powerlaw_leg(args, dev):
    """The power-law planted-community workload (8 M vertices, degree exponent
    2.5 in [8, 5000], community sizes exponent 1.5 in [20, 20000], mu 0.3,
    seed 3), generated on the device.  CPM(0.01) from singletons and WCC from
    the triangle-based start partition (-i 1), each through the driver loop
    with -s 2 (propagation, then merge).  Timed on the GPU: the first
    propagation sweep of each (CUDA events, repeated), the triangle count, the
    start partition and the whole schedule.  Checked on the host afterwards
    against the oracle's -p 1 schedule: every sweep's labels bit-exact, the
    contracted weights (a, b, w) of the final partition exact, the
    triangle counts exact, scores within 1e-12 (or the reference's own
    summation error bound)."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    import graphs
    import oracle
    import pcd

    t0 = time.time()
    ind, adj, _, _ = graphs.powerlaw_torch(args.pl_n, 2.5, 8, 5000, 1.5, 20, 20000, 0.3, seed=3, device=dev)
    torch.cuda.empty_cache()
    n, m = ind.shape[0] - 1, adj.shape[0] // 2
    log(f"[bench] power-law: n={n} m={m} ({time.time() - t0:.1f}s)")
    stream = torch.cuda.Stream(device=dev)
    ctx = pcd.Context(0)
    ctx.set_stream(stream.cuda_stream)
    out = {"workload": f"power-law planted communities n={args.pl_n} (degree exp 2.5 in [8, 5000], community exp "
                       f"1.5 in [20, 20000], mu 0.3, seed 3, device generator), degree-sorted",
           "n": int(n), "m": int(m), "max_degree": int(np.diff(ind).max())}
    gpu = {}
    for metric, init, iters in (("cpm-0.01", 0, args.pl_iters), ("wcc", 1, args.pl_wcc_iters)):
        rule = pcd.parse_metric(metric)
        G = pcd.Graph.from_csr(ctx, ind, adj)
        rec = {}
        if init == 1:
            torch.cuda.synchronize()
            t = time.perf_counter()
            G.count_triangles()
            rec["triangles_ms"] = 1000 * (time.perf_counter() - t)
            t = time.perf_counter()
            pcd.create_clustering_partition_device(G)
            rec["start_partition_ms"] = 1000 * (time.perf_counter() - t)
        else:
            G.labels = pcd.create_singleton_partition(G, pcd.GlibcRand(1))
        G.compress()
        start = torch.empty(n, dtype=torch.int32, device=dev)
        G.get_labels_device(start.data_ptr())
        seed1 = pcd.GlibcRand(1)
        if init == 0:
            seed1.skip(n)
        seed = seed1()
        ms = timed_sweeps(G, rule, start, seed, args.pl_reps + 1, stream)[1:]
        rec["sweep1_ms"] = statistics.median(ms)
        rec["sweep1_edges_per_s"] = m / (rec["sweep1_ms"] / 1e3)
        # the same sweep once more with CUDA events between the class launches
        try:
            ctx.profile(True)
            timed_sweeps(G, rule, start, seed, 1, stream)
            phases = {}
            for nm, t_ms in ctx.profile_read():  # a class may run as several launches
                if nm.startswith("sweep."):
                    phases[nm] = round(phases.get(nm, 0.0) + t_ms, 4)
            rec["sweep1_phases_ms"] = phases
        except Exception as e:  # the spans are a diagnostic: the leg goes on without them
            rec["sweep1_phases_ms"] = {"unavailable": str(e)[:200]}
        finally:
            ctx.profile(False)
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = pcd.run(G, rule, 2, 1.0, 1, iters, 0.0, init, keep_raw=True, initial_on_device=True)
        rec["schedule_s"] = time.perf_counter() - t
        rec["schedule"] = f"-m {metric} -s 2 -f 1.0 -n {iters} -i {init}"
        rec["score"] = res.score
        rec["k"] = res.k
        a, b, w = G.contract()
        tri = G.count_triangles()[:2] if init == 1 else None
        G.free()
        gpu[metric] = (rec, res, (a, b, w), tri)
        log(f"[bench] power-law {metric}: sweep 1 {rec['sweep1_ms']:.2f} ms, schedule {rec['schedule_s']:.2f} s")
    ctx.close()
    # the oracle checks, the two metrics side by side on host threads
    threads = os.cpu_count() or 1

    def check(metric, init, iters):
        rec, res, (a, b, w), tri = gpu[metric]
        port = oracle.Port()
        t = time.time()
        lab, score, sweeps = oracle.run_schedule(port, ind, adj, metric, 2, 1.0, 1, iters, 0.0, init,
                                                 aux_threads=max(1, threads - 2))
        diff = [int(np.count_nonzero(x.raw != y.raw)) for x, y in zip(res.log, sweeps)]
        st = port.stats(lab)
        ca, cb, cw = port.contract(lab, st)
        from_tol = abs(res.score - score) <= (1e-12 * abs(score) if metric == "wcc" else
                                              score_bound(metric, score, st, m))
        chk = {"sweeps_checked": len(diff), "labels_differing": diff,
               "bit_exact": len(res.log) == len(sweeps) and all(d == 0 for d in diff)
                            and np.array_equal(res.labels, lab),
               "contracted_pairs": int(len(ca)),
               "contracted_weights_exact": bool(np.array_equal(a, ca) and np.array_equal(b, cb)
                                                and np.array_equal(w, cw)),
               "score": res.score, "oracle_score": score, "score_within_tolerance": bool(from_tol),
               "oracle_seconds": round(time.time() - t, 1)}
        if tri is not None:
            chk["triangles_exact"] = bool(np.array_equal(tri[0], port.tri) and np.array_equal(tri[1], port.tri_deg))
        return metric, chk

    with ThreadPoolExecutor(2) as ex:
        checks = dict(ex.map(lambda c: check(*c), (("cpm-0.01", 0, args.pl_iters), ("wcc", 1, args.pl_wcc_iters))))
    for metric in gpu:
        out[metric] = gpu[metric][0] | {"parity": checks[metric]}
    log(f"[bench] power-law: {json.dumps(out)}")
    return out


def score_bound(metric, want, st, m):
    """1e-12 relative, or the reference's sequential FP64 sum's own rounding
    bound ((k + 3) 2^-53 sum |terms|) where larger (Modularity / CPM)."""
    import numpy as np

    import oracle

    rule, lam = oracle.parse_rule(metric)
    s = st.sizes.astype(np.float64)
    iv = st.int_volume.astype(np.float64)
    ev = st.ext_volume.astype(np.float64)
    if rule == 0:
        x = (iv + ev) / (2.0 * m)
        mag = float(np.sum(iv / (2.0 * m) + x * x))
    else:
        mag = float(np.sum(np.abs(iv) + lam * s * np.maximum(s - 1, 0))) / (2.0 * m)
    return max(1e-12 * abs(want), (len(s) + 3) * 2.0 ** -53 * mag)


def workload_config(args, n, m):
    return {
        "workload": f"rmat-s{args.scale}-ef{args.edge_factor} (a,b,c,d)=(.57,.19,.19,.05) seed 2, degree-sorted; "
                    f"Modularity refine sweeps 1-{args.sweeps} of the -s 0 schedule, cycled, frac 1.0",
        "n": int(n),
        "m": int(m),
        "sweep_bytes": int(16 * m + 12 * n + 4),
        "l2": "inputs larger than L2 (adjacency 8m bytes); L2 also flushed between steps (512 MiB write)",
        "parallelism": "replicas (one independent graph per GPU)",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--e2e-steps", type=int, default=5, help="e2e steps (cycling through the same sweeps)")
    ap.add_argument("--sweeps", type=int, default=5, help="cycle through the first S sweeps of the schedule")
    ap.add_argument("--bins", default="", help="degree classes, 7 comma-separated bounds (default: library's)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the timed sweeps")
    ap.add_argument("--tune", type=int, default=1, help="1: autotune degree classes and hub part size first")
    ap.add_argument("--batch-graphs", type=int, default=4096, help="0: skip the many-graph workload")
    ap.add_argument("--batch-reps", type=int, default=2)
    ap.add_argument("--batch-plain-stride", type=int, default=8)
    ap.add_argument("--batch-metric", default="mod")
    ap.add_argument("--batch-strategy", type=int, default=0)
    ap.add_argument("--batch-frac", type=float, default=0.5)
    ap.add_argument("--batch-iters", type=int, default=-1)
    ap.add_argument("--batch-threshold", type=float, default=0.0)
    ap.add_argument("--convert", type=int, default=1, help="0: skip the converter timing")
    ap.add_argument("--extras", type=int, default=1,
                    help="0: skip the components / NMI / initial-partition timings")
    ap.add_argument("--pl-n", type=int, default=8_000_000, help="power-law workload vertices (0: skip)")
    ap.add_argument("--pl-iters", type=int, default=4, help="CPM schedule iterations on the power-law graph")
    ap.add_argument("--pl-wcc-iters", type=int, default=2, help="WCC schedule iterations on the power-law graph")
    ap.add_argument("--pl-reps", type=int, default=5, help="timed repetitions of each first sweep")
    ap.add_argument("--serve-requests", type=int, default=600, help="0: skip the served workload")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[],
                    help="arrival rates (graphs/s); default: --serve-rate-multiples of the plain capacity")
    ap.add_argument("--serve-rate-multiples", type=float, nargs="+", default=[0.25, 1.0, 4.0, 16.0])
    ap.add_argument("--serve-iters", type=int, default=20, help="-n of every served request")
    ap.add_argument("--serve-seconds", type=float, default=15.0, help="arrival span per rate (bounds the requests)")
    ap.add_argument("--serve-workers", type=int, default=4)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        # NCCL between GPUs; gloo where there is no GPU (the reference arm on host cores)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    if args.impl == "reference":
        rc = run_reference_arm(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return rc

    import numpy as np

    import pcd

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ind, adj = make_workload(args, dev)
    n = ind.shape[0] - 1
    m = adj.shape[0] // 2

    stream = torch.cuda.Stream(device=dev)
    ctx = pcd.Context(local)
    ctx.set_stream(stream.cuda_stream)
    d_ind = torch.from_numpy(ind).to(dev)
    d_adj = torch.from_numpy(adj).to(dev)
    torch.cuda.synchronize()
    G = pcd.Graph.from_device(ctx, n, m, d_ind.data_ptr(), d_adj.data_ptr())
    rule = pcd.ModularityRule()
    tuning = None
    if args.bins:
        G.set_bins([int(x) for x in args.bins.split(",")])
    elif args.tune:
        import tune

        # degree classes and hub part size timed on this graph (outside the timed region)
        tr = tune.tune_graph(G, rule, cache_path=tune_cache(), retune=True, indices=ind)
        tuning = {k: tr[k] for k in ("bins", "hub_part", "ms", "default_ms", "signature")}
        tuning["candidates_timed"] = len(tr.get("timings", []))
        tuning["note"] = "ms: the schedule's first two sweeps, best tuned vs default classes"
        log(f"[bench] tuning: {json.dumps(tuning)}")
    sweep = pcd.PropagationRefinement(1.0)
    # The reference schedule (-s 0, frac 1.0): the start partition and rand_r
    # seed of each of its first S sweeps, kept on the device.
    seeds = schedule_seeds(ind, adj, args.sweeps)  # after create_singleton_partition's n draws
    starts = []
    G.set_labels_device(torch.arange(n, dtype=torch.int32, device=dev).data_ptr())
    for i in range(args.sweeps):
        G.compress()
        lab = torch.empty(n, dtype=torch.int32, device=dev)
        G.get_labels_device(lab.data_ptr())
        starts.append(lab)
        sweep.refine(G, rule, seeds[i])
    stream.synchronize()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    results = [None] * args.sweeps

    def step(i, ev0=None, ev1=None):
        j = i % args.sweeps
        with torch.cuda.stream(stream):
            flush.fill_(1)
            G.set_labels_device(starts[j].data_ptr())
            G.compress(sync=False)
            if ev0 is not None:
                ev0.record(stream)
            sweep.refine(G, rule, seeds[j])
            if ev1 is not None:
                ev1.record(stream)
        return j

    for i in range(max(3, args.warmup, args.sweeps)):
        j = step(i)
        stream.synchronize()
        results[j] = G.labels  # each sweep's result: checked against the oracle below

    k_before = G.info().kernels_total
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    for i, (e0, e1) in enumerate(evs):
        last = step(i, e0, e1)
    stream.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if dist:
        dist.barrier()
    sweep_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    launches = G.info().kernels_total - k_before
    total_ms = sum(sweep_ms)
    total_ms = max_over_ranks(dist, total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = world * m * args.steps / (total_ms / 1e3)
    assert np.array_equal(G.labels, results[last]), "sweep result changed between identical steps"

    # per-phase profile: every sweep of the cycle once more (events between
    # kernel groups), averaged, so that the classes add up to the timed mean
    # (the first sweep, from the singleton partition, differs from the rest)
    ctx.profile(True)
    phases = {}
    for i in range(args.sweeps):
        step(i)
        for nm, ms in ctx.profile_read():  # a class may run as several launches (degree sub-ranges)
            phases[nm] = phases.get(nm, 0.0) + ms / args.sweeps
    ctx.profile(False)
    info = G.info()
    bins_now = G.get_bins()
    peak, peak_kind = load_peaks()
    bb = bins_bytes(ind, bins_now[0])
    sweep_phases = {nm: ms for nm, ms in phases.items() if nm.startswith("sweep.")}
    dom = max(((nm, ms) for nm, ms in sweep_phases.items() if nm in bb), key=lambda x: x[1])
    dom_gbs = bb[dom[0]] / (dom[1] / 1e3) / 1e9
    sweep_bytes = 16 * m + 12 * n + 4
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(f"s{args.scale}", {}).get(dom[0])
    except Exception:
        pass

    # end to end through the C ABI with host buffers
    e2e = None
    if args.e2e_steps > 0:
        h_ind = torch.from_numpy(ind).pin_memory()
        h_adj = torch.from_numpy(adj).pin_memory()
        # the same cycle of sweeps as the resident steps: step i starts from
        # sweep (i mod S)'s start partition with that sweep's seed
        h_labs = [starts[j].cpu().pin_memory() for j in range(args.sweeps)]
        h_out = torch.empty(n, dtype=torch.int32).pin_memory()
        G.free()
        torch.cuda.empty_cache()

        def e2e_step(i, c=None, out=None, copy_lock=None, times=None):
            j = i % args.sweeps
            out = h_out if out is None else out
            t0 = time.perf_counter()
            if copy_lock is None:
                g2 = pcd.Graph.from_host_ptr(c or ctx, n, m, h_ind.data_ptr(), h_adj.data_ptr())
            else:
                with copy_lock:  # one copy over the host link at a time
                    g2 = pcd.Graph.from_host_ptr(c, n, m, h_ind.data_ptr(), h_adj.data_ptr())
            t1 = time.perf_counter()
            g2.set_labels_ptr(h_labs[j].data_ptr())
            sweep.refine(g2, rule, seeds[j])
            g2.get_labels_ptr(out.data_ptr())
            g2.free()
            if times is not None:
                times.append((t1 - t0, time.perf_counter() - t1))
            return j

        # Steps on W contexts at once, one host thread per context (as the
        # serving workers run), loads taken one at a time: while one graph is
        # copied from the host, the other context refines the previous one
        # (double buffering).  Step i runs on context i mod W; `check`
        # compares every step's labels with the resident run's.
        def e2e_run(steps, ctxs, check=False, times=None):
            outs = [torch.empty(n, dtype=torch.int32).pin_memory() for _ in ctxs]
            errors = []
            copy_lock = threading.Lock() if len(ctxs) > 1 else None

            def worker(w):
                try:
                    for i in range(w, steps, len(ctxs)):
                        j = e2e_step(i, ctxs[w], outs[w], copy_lock, times)
                        if check and not np.array_equal(outs[w].numpy(), results[j]):
                            raise AssertionError(f"end-to-end sweep {j} differs from the resident run")
                except BaseException as exc:  # re-raised on the main thread
                    errors.append(exc)

            threads = [threading.Thread(target=worker, args=(w,)) for w in range(len(ctxs))]
            t0 = time.perf_counter()
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            sec = time.perf_counter() - t0
            if errors:
                raise errors[0]
            return sec

        for i in range(args.sweeps):  # warm-up, and every sweep's labels against the resident run
            j = e2e_step(i)
            assert np.array_equal(h_out.numpy(), results[j]), f"end-to-end sweep {j} differs from the resident run"
        ctx2 = pcd.Context(local)
        pipe = [ctx, ctx2]
        e2e_run(2 * args.sweeps, pipe, check=True)  # warm-up of the second context, checked
        if dist:
            dist.barrier()
        sec_serial = e2e_run(args.e2e_steps, [ctx])
        if dist:
            dist.barrier()
        pipe_times = []
        sec = e2e_run(args.e2e_steps, pipe, times=pipe_times)
        sec = max_over_ranks(dist, sec, dev)
        sec_serial = max_over_ranks(dist, sec_serial, dev)
        e2e = {"value": world * m * args.e2e_steps / sec, "unit": "edges/s",
               "h2d_bytes_per_step": int(4 * (n + 1) + 8 * m + 4 * n), "d2h_bytes_per_step": int(4 * n),
               "ms_per_step": 1000.0 * sec / args.e2e_steps,
               "contexts": len(pipe),
               "pipelined_host_ms": {"load (copy lock held)": round(1000.0 * statistics.mean(t[0] for t in pipe_times), 3),
                                     "labels, refine, read-back, free": round(
                                         1000.0 * statistics.mean(t[1] for t in pipe_times), 3)},
               "serial": {"value": world * m * args.e2e_steps / sec_serial, "ms_per_step":
                          1000.0 * sec_serial / args.e2e_steps},
               "note": "each step: pcd_load_csr from pinned host CSR (validation, degree bins, buffers), "
                       "pcd_labels_set (the start partition of sweep i mod S), pcd_refine, pcd_labels_get, "
                       "pcd_graph_free; the same cycle of sweeps as value; steps on two contexts driven by "
                       "two host threads, one load at a time, so one step's copy overlaps the other's refine "
                       "(serial: one context)"}
        # where a step's time goes, averaged over one more cycle of the sweeps:
        # device spans of the load and of the refine call (CUDA events), host
        # time of the calls around them
        ctx.profile(True)
        ph = {}
        S = args.sweeps

        def add(key, sec):
            ph[key] = ph.get(key, 0.0) + sec / S

        for j in range(S):
            t0 = time.perf_counter()
            g2 = pcd.Graph.from_host_ptr(ctx, n, m, h_ind.data_ptr(), h_adj.data_ptr())
            add("load (host)", time.perf_counter() - t0)
            for nm, ms in ctx.profile_read():
                add(nm, ms / 1000.0)
            t0 = time.perf_counter()
            g2.set_labels_ptr(h_labs[j].data_ptr())
            add("labels_set (host)", time.perf_counter() - t0)
            t0 = time.perf_counter()
            sweep.refine(g2, rule, seeds[j])
            ctx.synchronize()
            add("refine (host)", time.perf_counter() - t0)
            for nm, ms in ctx.profile_read():
                add("refine." + nm if nm == "compress" or nm.startswith("stats") else "refine.sweep", ms / 1000.0)
            t0 = time.perf_counter()
            g2.get_labels_ptr(h_out.data_ptr())
            add("labels_get (host)", time.perf_counter() - t0)
            t0 = time.perf_counter()
            g2.free()
            add("free (host)", time.perf_counter() - t0)
        ctx.profile(False)
        e2e["phases_ms"] = {k: round(1000.0 * v, 3) for k, v in ph.items()}
        ctx2.close()

    batched = batched_s2 = None
    if args.batch_graphs > 0:
        del d_ind, d_adj
        torch.cuda.empty_cache()
        batched = batched_leg(args, ctx, dev)
        torch.cuda.empty_cache()
        # alternating propagation and merging: merge iterations in the timed region
        batched_s2 = batched_leg(args, ctx, dev, strategy=2, frac=1.0)

    converted = None
    if args.convert:
        torch.cuda.empty_cache()
        converted = convert_leg(args, dev, ind, adj)

    extras = None
    if args.extras:
        torch.cuda.empty_cache()
        extras = extras_leg(args, dev, ind, adj)

    powerlaw = None
    if args.pl_n > 0:
        torch.cuda.empty_cache()
        powerlaw = powerlaw_leg(args, dev)

    served = None
    if args.serve_requests > 0:
        torch.cuda.empty_cache()
        served = served_leg(args, dev)

    parity = None
    if rank == 0 and not args.no_parity:
        h_starts = [x.cpu().numpy() for x in starts]
        parity = oracle_sweep_parity(ind, adj, h_starts, seeds, results, 600.0)
        log(f"[bench] parity: {json.dumps(parity)}")

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, k, sec = cpu_sweeps(ind, adj, seeds, threads, args.sweeps, 30.0)
        cpu = {"value": v, "unit": "edges/s", "cores": threads, "kind": "port",
               "sample": f"{k} propagation sweep(s) (the schedule's first, in order) of the workload graph, "
                         f"oracle OpenMP restatement of PropagationRefinement::refine, {threads} threads, "
                         f"{sec:.1f}s"}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "edges/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(3, args.warmup),
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int32 labels / int64 exact gain keys (fp64 recheck)",
            "data": "synthetic",
            "config": workload_config(args, n, m),
            "roofline": {"bound": "hbm", "kernel": dom[0], "achieved": dom_gbs, "peak": peak, "unit": "GB/s",
                         "frac": dom_gbs / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": bb[dom[0]], "launch_ms": dom[1],
                         "sweep_achieved": sweep_bytes / (ms_per_step / 1e3) / 1e9,
                         "sweep_frac": sweep_bytes / (ms_per_step / 1e3) / 1e9 / peak},
            "cpu_baseline": cpu,
            "parity": parity,
            "e2e": e2e,
            "batched": batched,
            "batched_s2": batched_s2,
            "served": served,
            "powerlaw": powerlaw,
            "convert": converted,
            "extras": extras,
            "gpu_launches": int(launches),
            "clocks": clk,
            "phases_ms": {nm: round(ms, 4) for nm, ms in phases.items()},
            "phases_over": f"mean of the cycle's {args.sweeps} sweeps (CUDA events between kernel groups)",
            "per_sweep_ms": [round(statistics.mean(sweep_ms[j::args.sweeps]), 3)
                             for j in range(min(args.sweeps, len(sweep_ms)))],
            "bins": bins_now,
            "tuning": tuning,
            "sweep_info": {"draws": info.draws, "fp64_recheck_vertices": info.fallback,
                           "tie_replays": info.resolved},
            "wall_s_timed": wall,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
