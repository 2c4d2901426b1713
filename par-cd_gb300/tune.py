"""Autotuner of the sweep's launch configuration (no counterpart in the
reference, whose GPU path sorts every edge in one pass).

What it moves: the degree classes (pcd_graph_set_bins: where the warp, block,
large-block and hub kernels take over, which also sizes each class's
shared-memory tables and block shapes, since those follow a sub-range's
largest degree) and the hub kernel's hash-part size (pcd_graph_set_hub_part).
Results never depend on either; only time does.

How: every candidate is timed on the graph itself over a fixed set of
propagation sweeps (the first two sweeps of the reference schedule from the
singleton partition, each from its own start partition), best of `reps`; the
bounds are searched first, then the part size for the best bounds.  The
winner is stored in a JSON file keyed by a signature of the degree
distribution (the share of adjacency entries per power-of-two degree range,
and the scale of the edge count), so that graphs of the same shape reuse it
without timing anything.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

DEFAULT_BINS = [4, 8, 16, 32, 256, 2048, 8192]
DEFAULT_HUB_PART = 6144


def default_cache_path() -> str:
    return os.environ.get("PCD_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "par-cd_gb300",
                                                         "tuning.json"))


def signature(indices) -> str:
    """Degree-distribution key: log2 of the edge count, then the share of
    adjacency entries (in 1/32 steps) in each degree range (2^i, 2^(i+1)]."""
    deg = np.diff(np.asarray(indices, dtype=np.int64))
    tot = max(1, int(deg.sum()))
    cls = np.zeros(33, np.int64)
    nz = deg[deg > 0]
    np.add.at(cls, np.ceil(np.log2(nz)).astype(np.int64), nz)
    share = np.rint(32.0 * cls / tot).astype(np.int64)
    last = int(np.max(np.nonzero(share)[0])) if share.any() else 0
    return f"m2^{int(round(np.log2(max(1, tot // 2))))}:" + ".".join(str(int(x)) for x in share[:last + 1])


def candidate_bins():
    """Valid bound sets around the defaults (thread classes fixed)."""
    out = []
    for warp in (128, 256):
        for block in (512, 1024, 2048):
            for large in sorted({block, 4096, 8192}):
                out.append([4, 8, 16, 32, warp, block, large])
    return out


def load_cache(path: str | None = None) -> dict:
    path = path or default_cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(entries: dict, path: str | None = None):
    path = path or default_cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(entries, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def search(apply, run_once, reps: int = 2, bins=None, parts=(4096, 6144, 8192)) -> dict:
    """Times `run_once` (which returns seconds) under every candidate that
    `apply(bins, hub_part)` installs; returns the best configuration and the
    timings.  The configuration left installed is the best one."""
    bins = bins or candidate_bins()
    timings = []

    def timed(b, p):
        apply(b, p)
        best = min(run_once() for _ in range(reps))
        timings.append({"bins": list(b), "hub_part": int(p), "ms": 1000.0 * best})
        return best

    base = timed(DEFAULT_BINS, DEFAULT_HUB_PART)
    best_b, best_t = DEFAULT_BINS, base
    for b in bins:
        if b == DEFAULT_BINS:
            continue
        t = timed(b, DEFAULT_HUB_PART)
        if t < best_t:
            best_b, best_t = b, t
    best_p = DEFAULT_HUB_PART
    for p in parts:
        if p == DEFAULT_HUB_PART:
            continue
        t = timed(best_b, p)
        if t < best_t:
            best_p, best_t = p, t
    apply(best_b, best_p)
    return {"bins": list(best_b), "hub_part": int(best_p), "ms": 1000.0 * best_t, "default_ms": 1000.0 * base,
            "timings": timings}


def tune_graph(G, rule, cache_path: str | None = None, reps: int = 2, retune: bool = False,
               indices=None) -> dict:
    """Tunes a single graph (pcd.Graph) for `rule`, or applies the stored
    configuration of its signature.  `indices`: the graph's host row offsets
    when the caller has them (else they are read back).  Returns the entry
    (with "cached": True when nothing was timed)."""
    import pcd

    ind = indices if indices is not None else (G._indices if G._indices is not None else G.csr()[0])
    key = f"{signature(ind)}|rule{rule.kind}"
    entries = load_cache(cache_path)
    if key in entries and not retune:
        e = entries[key]
        G.set_bins(e["bins"])
        G.set_hub_part(e["hub_part"])
        return dict(e, cached=True, signature=key)
    # the schedule's first two propagation sweeps from the singleton partition
    rand = pcd.GlibcRand(1)
    G.labels = pcd.create_singleton_partition(G, rand)
    starts, seeds = [], []
    sweep = pcd.PropagationRefinement(1.0)
    for _ in range(2):
        G.compress()
        starts.append(G.labels)
        seeds.append(rand())
        sweep.refine(G, rule, seeds[-1])

    def run_once():
        total = 0.0
        for lab, sd in zip(starts, seeds):
            G.labels = lab
            G.compress()
            G.ctx.synchronize()
            t0 = time.perf_counter()
            sweep.refine(G, rule, sd)
            G.ctx.synchronize()
            total += time.perf_counter() - t0
        return total

    def apply(b, p):
        G.set_bins(b)
        G.set_hub_part(p)

    res = search(apply, run_once, reps)
    entry = {"bins": res["bins"], "hub_part": res["hub_part"], "ms": res["ms"], "default_ms": res["default_ms"]}
    entries = load_cache(cache_path)
    entries[key] = entry
    save_cache(entries, cache_path)
    return dict(entry, cached=False, signature=key, timings=res["timings"])


def tune_batch(B, rule, frac: float, indices, cache_path: str | None = None, reps: int = 2,
               retune: bool = False) -> dict:
    """Tunes a batch (pcd.Batch) on its first propagation step from
    singletons (each graph with its own first seed, frac as in its schedule),
    or applies the stored configuration of the union's degree signature.
    `indices`: the union's host row offsets."""
    import pcd

    key = f"batch|{signature(indices)}|rule{rule.kind}|f{frac}"
    entries = load_cache(cache_path)
    if key in entries and not retune:
        e = entries[key]
        B.set_bins(e["bins"])
        B.set_hub_part(e["hub_part"])
        return dict(e, cached=True, signature=key)
    sizes = np.diff(B.voff)
    seeds = np.empty(B.G, np.uint32)
    for g, n in enumerate(sizes):
        r = pcd.GlibcRand(1)
        r.skip(int(n))
        seeds[g] = r()
    start = np.concatenate([np.arange(n, dtype=np.int32) for n in sizes]) if B.G else np.zeros(0, np.int32)

    def run_once():
        B.labels = start
        B.compress()
        B.ctx.synchronize()
        t0 = time.perf_counter()
        B.refine(rule, frac, seeds)
        B.ctx.synchronize()
        return time.perf_counter() - t0

    def apply(b, p):
        B.set_bins(b)
        B.set_hub_part(p)

    res = search(apply, run_once, reps)
    entry = {"bins": res["bins"], "hub_part": res["hub_part"], "ms": res["ms"], "default_ms": res["default_ms"]}
    entries = load_cache(cache_path)
    entries[key] = entry
    save_cache(entries, cache_path)
    return dict(entry, cached=False, signature=key, timings=res["timings"])
