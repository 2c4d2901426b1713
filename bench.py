#!/usr/bin/env python
"""Benchmark of the refine sweep (the headline of this repository).

Workload (N=1): R-MAT scale 24, edge factor 16, quadrants (.57, .19, .19, .05),
seed 2, random vertex permutation, loops/duplicates/isolated vertices removed
and vertices renumbered by decreasing degree as the reference converter does.
One step = one synchronous label-propagation sweep with the Modularity rule,
frac 1.0, from the singleton partition (the reference's first sweep: compress
+ statistics are done before the timed sweep of every step, from the same
start partition and the same rand_r seed).

Lines printed (rank 0, one JSON line):
  value      refine-sweep edges/s, inputs resident in HBM, CUDA events on the
             stream the kernels run on, max over ranks
  e2e        the same metric through the C ABI with HOST buffers: every step
             loads the CSR from pinned host memory, sets the start labels,
             sweeps, and reads the labels back
  roofline   the sweep's dominant kernel against the measured HBM copy peak
  cpu_baseline  the oracle (C restatement of the reference, OpenMP) on the
             host cores, on the same graph
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


def bins_bytes(ind):
    """Algorithmic bytes per vertex class: 8 deg + 12 (row offsets, adjacency,
    neighbour-label gathers, own label read, new label write)."""
    import numpy as np

    deg = np.diff(ind.astype(np.int64))
    edges = [0, 4, 8, 16, 32, 256, 2048, 8192, 1 << 62]
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


def schedule_seeds(n, count):
    import pcd

    r = pcd.GlibcRand()
    r.skip(n)
    return [r() for _ in range(count)]


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    import torch

    dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    ind, adj = make_workload(args, dev)
    n = ind.shape[0] - 1
    m = adj.shape[0] // 2
    seeds = schedule_seeds(n, args.sweeps)
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
                                   f"PropagationRefinement::refine on {threads} host threads, {sec:.1f}s"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--sweeps", type=int, default=5, help="cycle through the first S sweeps of the schedule")
    ap.add_argument("--bins", default="", help="degree classes, 7 comma-separated bounds (default: library's)")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

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
    if args.bins:
        G.set_bins([int(x) for x in args.bins.split(",")])
    rule = pcd.ModularityRule()
    sweep = pcd.PropagationRefinement(1.0)
    # The reference schedule (-s 0, frac 1.0): the start partition and rand_r
    # seed of each of its first S sweeps, kept on the device.
    seeds = schedule_seeds(n, args.sweeps)  # after create_singleton_partition's n draws
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
        results[j] = G.labels  # each sweep's result, for a self-consistency check below

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
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * m * args.steps / (total_ms / 1e3)
    assert np.array_equal(G.labels, results[last]), "sweep result changed between identical steps"

    # per-phase profile of one more step (events between kernel groups)
    ctx.profile(True)
    step(0)
    phases = ctx.profile_read()
    ctx.profile(False)
    info = G.info()
    bins_now = G.get_bins()
    peak, peak_kind = load_peaks()
    bb = bins_bytes(ind)
    sweep_phases = {nm: ms for nm, ms in phases if nm.startswith("sweep.")}
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
        h_lab = starts[0].cpu().pin_memory()
        h_out = torch.empty(n, dtype=torch.int32).pin_memory()
        G.free()
        torch.cuda.empty_cache()

        def e2e_step():
            g2 = pcd.Graph.from_host_ptr(ctx, n, m, h_ind.data_ptr(), h_adj.data_ptr())
            g2.set_labels_ptr(h_lab.data_ptr())
            sweep.refine(g2, rule, seeds[0])
            g2.get_labels_ptr(h_out.data_ptr())
            g2.free()

        e2e_step()
        assert np.array_equal(h_out.numpy(), results[0]), "end-to-end result differs from the resident run"
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        sec = time.perf_counter() - t0
        if dist:
            t = torch.tensor([sec], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            sec = float(t.item())
        e2e = {"value": world * m * args.e2e_steps / sec, "unit": "edges/s",
               "h2d_bytes_per_step": int(4 * (n + 1) + 8 * m + 4 * n), "d2h_bytes_per_step": int(4 * n),
               "ms_per_step": 1000.0 * sec / args.e2e_steps,
               "note": "each step: pcd_load_csr from pinned host CSR (validation, degree bins, buffers), "
                       "pcd_labels_set, pcd_refine, pcd_labels_get, pcd_graph_free"}

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
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "phases_ms": {nm: round(ms, 4) for nm, ms in phases},
            "per_sweep_ms": [round(statistics.mean(sweep_ms[j::args.sweeps]), 3) for j in range(args.sweeps)],
            "bins": bins_now,
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
