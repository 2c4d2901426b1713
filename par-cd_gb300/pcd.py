"""Python host side of libpcd: the reference's phase and rule interfaces
(src/framework.hpp:8-11, src/rules.hpp:9-19, src/refinement.hpp:8-42, the GPU
host API src/framework-cuda.cuh:14-23) over the C ABI in include/pcd.h.

Every call goes through libpcd.so; there is no CPU path.  If the library
cannot be loaded the import of this module raises.

    ctx = Context(0)
    g = Graph.from_csr(ctx, indices, adj)
    rand = GlibcRand()                          # the reference's rand() stream
    g.labels = create_singleton_partition(g, rand)
    k = g.compress()                            # compress_labels + collect_statistics
    score = ModularityRule().calculate(g)
    PropagationRefinement(1.0).refine(g, ModularityRule(), rand())
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpcd.so")

NEW_LABEL = -1


class PcdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class _Rule(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lam", C.c_double)]


class _Info(C.Structure):
    _fields_ = [("draws", C.c_int64), ("fallback", C.c_int32), ("resolved", C.c_int32),
                ("kernels", C.c_int32), ("merge_pairs", C.c_int32), ("kernels_total", C.c_int64)]


class _Rand(C.Structure):
    _fields_ = [("r", C.c_uint32 * 34), ("pos", C.c_int32)]


class _Schedule(C.Structure):
    _fields_ = [("rule", _Rule), ("strategy", C.c_int32), ("frac", C.c_double), ("rounds", C.c_int32),
                ("n_iter", C.c_int32), ("threshold", C.c_double)]


class _ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("workers", C.c_int32), ("max_batch_graphs", C.c_int32),
                ("max_batch_edges", C.c_int64), ("hbm_budget_bytes", C.c_int64), ("max_wait_ms", C.c_double),
                ("use_cuda_graph", C.c_int32), ("small_graph_edges", C.c_int64), ("large_graph_edges", C.c_int64),
                ("continuous", C.c_int32)]


class _ServeStats(C.Structure):
    _fields_ = [(nm, C.c_int64) for nm in ("submitted", "completed", "failed", "batches", "batched_graphs",
                                           "queue_len", "bytes_in_flight", "bytes_peak", "bytes_measured_peak",
                                           "estimate_exceeded", "admitted_running", "released_early")]


class _ServeTiming(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("latency_ms", C.c_double), ("batch_graphs", C.c_int64)]


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libpcd.so is not built ({LIB_PATH}); run par-cd_gb300/build.py")
    lib = C.CDLL(LIB_PATH)
    vp, i32, i64, u32, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
    sig = {
        "pcd_status_string": ([i32], C.c_char_p),
        "pcd_last_error": ([vp], C.c_char_p),
        "pcd_init": ([C.POINTER(vp), i32], i32),
        "pcd_destroy": ([vp], i32),
        "pcd_set_stream": ([vp, vp], i32),
        "pcd_synchronize": ([vp], i32),
        "pcd_set_class_streams": ([vp, i32], i32),
        "pcd_load_csr": ([vp, i32, i32, vp, vp, C.POINTER(vp)], i32),
        "pcd_load_csr_device": ([vp, i32, i32, vp, vp, C.POINTER(vp)], i32),
        "pcd_graph_free": ([vp], i32),
        "pcd_labels_set": ([vp, vp], i32),
        "pcd_labels_get": ([vp, vp], i32),
        "pcd_labels_set_device": ([vp, vp], i32),
        "pcd_labels_get_device": ([vp, vp], i32),
        "pcd_compress": ([vp, C.POINTER(i32)], i32),
        "pcd_stats_get": ([vp, vp, vp, vp], i32),
        "pcd_triangles": ([vp, vp, vp, C.POINTER(dbl)], i32),
        "pcd_score": ([vp, C.POINTER(_Rule), C.POINTER(dbl)], i32),
        "pcd_refine": ([vp, C.POINTER(_Rule), dbl, u32], i32),
        "pcd_merge": ([vp, C.POINTER(_Rule), i32, u32], i32),
        "pcd_contract": ([vp, i64, vp, vp, vp, C.POINTER(i64)], i32),
        "pcd_sweep_info_get": ([vp, C.POINTER(_Info)], i32),
        "pcd_profile_enable": ([vp, i32], i32),
        "pcd_graph_set_bins": ([vp, C.POINTER(i32)], i32),
        "pcd_graph_get_bins": ([vp, C.POINTER(i32), C.POINTER(i64)], i32),
        "pcd_graph_set_hub_part": ([vp, i32], i32),
        "pcd_profile_read": ([vp, C.POINTER(C.c_char_p), C.POINTER(dbl), i32], i32),
        "pcd_batch_load": ([vp, i32, vp, vp, vp, C.POINTER(vp)], i32),
        "pcd_batch_load_device": ([vp, i32, vp, vp, vp, C.POINTER(vp)], i32),
        "pcd_batch_num_graphs": ([vp, C.POINTER(i32)], i32),
        "pcd_batch_labels_set": ([vp, vp], i32),
        "pcd_batch_labels_get": ([vp, vp], i32),
        "pcd_batch_compress": ([vp, vp], i32),
        "pcd_batch_score": ([vp, C.POINTER(_Rule), vp], i32),
        "pcd_batch_refine": ([vp, C.POINTER(_Rule), dbl, vp], i32),
        "pcd_batch_merge": ([vp, C.POINTER(_Rule), i32, vp], i32),
        "pcd_batch_run": ([vp, C.POINTER(_Rule), i32, dbl, i32, i32, dbl, i32, vp, vp], i32),
        "pcd_compress_labels_noalloc": ([vp, i32, vp, vp, vp], i32),
        "pcd_graph_device_bytes": ([vp, C.POINTER(i64)], i32),
        "pcd_convert_edges": ([vp, i64, vp, vp, i32, vp, C.POINTER(vp)], i32),
        "pcd_graph_size": ([vp, C.POINTER(i32), C.POINTER(i32)], i32),
        "pcd_graph_csr_get": ([vp, vp, vp], i32),
        "pcd_estimate_device_bytes": ([i32, i64, i32, i64, i32, i32, i32, i32, C.POINTER(i64)], i32),
        "pcd_device_sm_count": ([vp, C.POINTER(i32)], i32),
        "pcd_serve_start": ([C.POINTER(_ServeConfig), C.POINTER(vp)], i32),
        "pcd_serve_submit": ([vp, i32, i32, vp, vp, C.POINTER(_Schedule), C.POINTER(C.c_uint64)], i32),
        "pcd_serve_poll": ([vp, C.c_uint64, C.POINTER(i32)], i32),
        "pcd_serve_wait": ([vp, C.c_uint64, vp, C.POINTER(dbl), C.POINTER(i32), C.POINTER(_ServeTiming)], i32),
        "pcd_serve_stats_get": ([vp, C.POINTER(_ServeStats)], i32),
        "pcd_serve_stop": ([vp], i32),
        "pcd_rand_seed": ([C.POINTER(_Rand), u32], None),
        "pcd_rand_next": ([C.POINTER(_Rand)], i32),
        "pcd_rand_skip": ([C.POINTER(_Rand), i64], None),
        "pcd_singleton_partition": ([C.POINTER(_Rand), i32, vp], i32),
        "pcd_clustering_partition": ([i32, vp, vp, vp, vp], i32),
        "pcd_clustering_partition_device": ([vp, C.POINTER(i32)], i32),
        "pcd_find_connected": ([vp, C.POINTER(i32)], i32),
        "pcd_nmi_device": ([vp, i64, vp, vp, i32, C.POINTER(dbl)], i32),
        "pcd_nmi": ([vp, i64, vp, vp, i32, C.POINTER(dbl)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


LIB = _load()


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None and a.size else C.c_void_p(0)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------------------
# rules (src/rules.hpp)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Rule:
    kind: int
    lam: float = 0.0

    def _c(self) -> _Rule:
        return _Rule(self.kind, self.lam)

    def calculate(self, g: "Graph") -> float:
        """Rule::calculate on the graph's current partition (FP64)."""
        out = C.c_double()
        g.ctx._check(LIB.pcd_score(g.h, C.byref(self._c()), C.byref(out)))
        return out.value

    def get_name(self) -> str:
        return {0: "modularity", 1: f"CPM (lambda={self.lam:g})", 2: "WCC"}[self.kind]


def ModularityRule() -> Rule:
    return Rule(0)


def CPMRule(lam: float) -> Rule:
    return Rule(1, float(lam))


def WCCRule() -> Rule:
    return Rule(2)


def parse_metric(spec: str) -> Rule:
    """-m mod | wcc | cpm-<gamma> (src/main.cpp:125-141)."""
    s = spec.lower()
    if s in ("mod", "modularity"):
        return ModularityRule()
    if s == "wcc":
        return WCCRule()
    if s.startswith("cpm-") and len(s) > 4:
        return CPMRule(float(s[4:]))
    raise ValueError(f"unknown metric: {spec}")


# ---------------------------------------------------------------------------
# context / graph
# ---------------------------------------------------------------------------
class Context:
    """cuda_init / cuda_deinit (src/framework-cuda.cu:59-78)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = LIB.pcd_init(C.byref(h), device)
        self.h = h
        if st != 0:
            msg = LIB.pcd_last_error(h).decode() if h else ""
            if h:
                LIB.pcd_destroy(h)
            self.h = None
            raise PcdError(st, f"pcd_init({device}) failed: {msg}")
        self.device = device

    def _check(self, st: int):
        if st != 0:
            msg = LIB.pcd_last_error(self.h).decode() if self.h else ""
            raise PcdError(st, f"{LIB.pcd_status_string(st).decode()}: {msg}")

    def set_stream(self, stream_ptr: int | None):
        self._check(LIB.pcd_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    def class_streams(self, on: bool = True):
        """Run a sweep's degree classes concurrently on side streams."""
        self._check(LIB.pcd_set_class_streams(self.h, 1 if on else 0))

    def synchronize(self):
        self._check(LIB.pcd_synchronize(self.h))

    def profile(self, on: bool = True):
        self._check(LIB.pcd_profile_enable(self.h, 1 if on else 0))

    def profile_read(self) -> list:
        names = (C.c_char_p * 64)()
        ms = (C.c_double * 64)()
        k = LIB.pcd_profile_read(self.h, names, ms, 64)
        if k < 0:
            raise PcdError(2, "pcd_profile_read failed")
        return [(names[i].decode(), ms[i]) for i in range(min(k, 64))]

    def close(self):
        if self.h:
            LIB.pcd_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclass
class SweepInfo:
    draws: int
    fallback: int
    resolved: int
    kernels: int
    merge_pairs: int
    kernels_total: int


class Graph:
    """A graph resident on the device with its current partition
    (Graph src/graph.hpp:6-40 + Partition src/common.hpp:26-37)."""

    def __init__(self, ctx: Context, h, n: int, m: int, indices=None, adj=None):
        self.ctx, self.h, self.n, self.m = ctx, h, n, m
        self._indices, self._adj = indices, adj

    @classmethod
    def from_csr(cls, ctx: Context, indices, adj) -> "Graph":
        """cuda_transfer_graph from host CSR arrays."""
        ind = _i32(indices)
        a = _i32(adj)
        n = ind.shape[0] - 1
        m = a.shape[0] // 2
        h = C.c_void_p()
        ctx._check(LIB.pcd_load_csr(ctx.h, n, m, _ptr(ind), _ptr(a), C.byref(h)))
        return cls(ctx, h, n, m, ind, a)

    @classmethod
    def from_host_ptr(cls, ctx: Context, n: int, m: int, indices_ptr: int, adj_ptr: int) -> "Graph":
        """Load from raw host pointers (e.g. pinned buffers)."""
        h = C.c_void_p()
        ctx._check(LIB.pcd_load_csr(ctx.h, n, m, C.c_void_p(indices_ptr), C.c_void_p(adj_ptr), C.byref(h)))
        return cls(ctx, h, n, m)

    @classmethod
    def from_device(cls, ctx: Context, n: int, m: int, d_indices: int, d_adj: int) -> "Graph":
        h = C.c_void_p()
        ctx._check(LIB.pcd_load_csr_device(ctx.h, n, m, C.c_void_p(d_indices), C.c_void_p(d_adj), C.byref(h)))
        return cls(ctx, h, n, m)

    def free(self):
        if self.h:
            LIB.pcd_graph_free(self.h)
            self.h = None

    # labels -------------------------------------------------------------
    @property
    def labels(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        self.ctx._check(LIB.pcd_labels_get(self.h, _ptr(out)))
        return out

    @labels.setter
    def labels(self, lab):
        lab = _i32(lab)
        if lab.shape[0] != self.n:
            raise ValueError("labels must have n entries")
        self.ctx._check(LIB.pcd_labels_set(self.h, _ptr(lab)))

    def set_labels_ptr(self, host_ptr: int):
        self.ctx._check(LIB.pcd_labels_set(self.h, C.c_void_p(host_ptr)))

    def get_labels_ptr(self, host_ptr: int):
        self.ctx._check(LIB.pcd_labels_get(self.h, C.c_void_p(host_ptr)))

    def set_labels_device(self, ptr: int):
        self.ctx._check(LIB.pcd_labels_set_device(self.h, C.c_void_p(ptr)))

    def get_labels_device(self, ptr: int):
        self.ctx._check(LIB.pcd_labels_get_device(self.h, C.c_void_p(ptr)))

    # phases -------------------------------------------------------------
    def compress(self, sync: bool = True) -> int | None:
        """compress_labels + collect_statistics; returns the community count."""
        if not sync:
            self.ctx._check(LIB.pcd_compress(self.h, None))
            return None
        k = C.c_int32()
        self.ctx._check(LIB.pcd_compress(self.h, C.byref(k)))
        return k.value

    def stats(self):
        k = self.compress()
        s = np.zeros(max(k, 1), np.int32)
        i = np.zeros(max(k, 1), np.int32)
        e = np.zeros(max(k, 1), np.int32)
        self.ctx._check(LIB.pcd_stats_get(self.h, _ptr(s), _ptr(i), _ptr(e)))
        return s[:k], i[:k], e[:k]

    def count_triangles(self):
        tri = np.zeros(self.n, np.int32)
        td = np.zeros(self.n, np.int32)
        cc = C.c_double()
        self.ctx._check(LIB.pcd_triangles(self.h, _ptr(tri), _ptr(td), C.byref(cc)))
        return tri, td, cc.value

    def contract(self):
        """Contracted edge weights (a, b, w), sorted by (a, b)."""
        npairs = C.c_int64()
        self.ctx._check(LIB.pcd_contract(self.h, 0, None, None, None, C.byref(npairs)))
        P = npairs.value
        a = np.zeros(max(P, 1), np.int32)
        b = np.zeros(max(P, 1), np.int32)
        w = np.zeros(max(P, 1), np.int32)
        self.ctx._check(LIB.pcd_contract(self.h, P, _ptr(a), _ptr(b), _ptr(w), C.byref(npairs)))
        return a[:P], b[:P], w[:P]

    def csr(self):
        """The graph's CSR as host arrays (indices[n + 1], adj[2m])."""
        ind = np.empty(self.n + 1, np.int32)
        adj = np.empty(max(2 * self.m, 1), np.int32)
        self.ctx._check(LIB.pcd_graph_csr_get(self.h, _ptr(ind), _ptr(adj)))
        return ind, adj[: 2 * self.m]

    def set_bins(self, max_deg):
        arr = (C.c_int32 * 7)(*[int(x) for x in max_deg])
        self.ctx._check(LIB.pcd_graph_set_bins(self.h, arr))

    def set_hub_part(self, labels: int):
        """Distinct labels per hash part of the hub kernel."""
        self.ctx._check(LIB.pcd_graph_set_hub_part(self.h, int(labels)))

    def get_bins(self):
        md = (C.c_int32 * 7)()
        cnt = (C.c_int64 * 8)()
        self.ctx._check(LIB.pcd_graph_get_bins(self.h, md, cnt))
        return list(md), list(cnt)

    def info(self) -> SweepInfo:
        i = _Info()
        self.ctx._check(LIB.pcd_sweep_info_get(self.h, C.byref(i)))
        return SweepInfo(i.draws, i.fallback, i.resolved, i.kernels, i.merge_pairs, i.kernels_total)


# ---------------------------------------------------------------------------
# refinements (src/refinement.hpp)
# ---------------------------------------------------------------------------
class PropagationRefinement:
    def __init__(self, frac: float):
        self.frac = float(frac)

    def refine(self, g: Graph, rule: Rule, seed: int):
        g.ctx._check(LIB.pcd_refine(g.h, C.byref(rule._c()), self.frac, C.c_uint32(seed & 0xFFFFFFFF)))


class MergingRefinement:
    def __init__(self, rounds: int = 1):
        self.rounds = int(rounds)

    def refine(self, g: Graph, rule: Rule, seed: int):
        g.ctx._check(LIB.pcd_merge(g.h, C.byref(rule._c()), self.rounds, C.c_uint32(seed & 0xFFFFFFFF)))


class FindConnectedRefinement:
    """FindConnectedRefinement (src/refinement.cpp:291-322): every vertex's
    label becomes the smallest vertex id of its connected component."""

    def __init__(self, num_threads: int = 1):
        self.num_threads = num_threads  # the reference's OpenMP width; unused here

    def refine(self, g: Graph, rule: Rule | None = None, seed: int = 0) -> int:
        k = C.c_int32()
        g.ctx._check(LIB.pcd_find_connected(g.h, C.byref(k)))
        return int(k.value)


class GlibcRand:
    """The reference's rand() stream (glibc, default seed 1)."""

    def __init__(self, seed: int = 1):
        self._s = _Rand()
        LIB.pcd_rand_seed(C.byref(self._s), seed)

    def __call__(self) -> int:
        return int(LIB.pcd_rand_next(C.byref(self._s)))

    def skip(self, count: int):
        LIB.pcd_rand_skip(C.byref(self._s), count)


def create_singleton_partition(g: Graph, rand: GlibcRand) -> np.ndarray:
    lab = np.zeros(g.n, np.int32)
    g.ctx._check(LIB.pcd_singleton_partition(C.byref(rand._s), g.n, _ptr(lab)))
    return lab


def create_clustering_partition(g: Graph) -> np.ndarray:
    tri, _, _ = g.count_triangles()
    if g._indices is None:
        raise ValueError("clustering partition needs the host CSR")
    lab = np.zeros(g.n, np.int32)
    g.ctx._check(LIB.pcd_clustering_partition(g.n, _ptr(g._indices), _ptr(g._adj), _ptr(tri), _ptr(lab)))
    return lab


def create_clustering_partition_device(g: Graph) -> int:
    """create_clustering_partition (src/framework.cpp:27-59) computed on the
    device into the graph's labels; returns the number of communities."""
    k = C.c_int32()
    g.ctx._check(LIB.pcd_clustering_partition_device(g.h, C.byref(k)))
    return int(k.value)


def nmi(ctx: Context, a, b, n: int | None = None) -> float:
    """norm_mutual_info (src/common.cpp:75-125) of the label pairs (a[i],
    b[i]), normalised by n (default len(a)).  a and b: host arrays, or CUDA
    tensors / objects with data_ptr() (device arrays, not copied)."""
    out = C.c_double()
    if hasattr(a, "data_ptr"):
        count = int(a.numel())
        ctx._check(LIB.pcd_nmi_device(ctx.h, count, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                      count if n is None else n, C.byref(out)))
    else:
        x, y = _i32(a), _i32(b)
        if x.shape != y.shape:
            raise ValueError("labelings differ in length")
        count = int(x.shape[0])
        ctx._check(LIB.pcd_nmi(ctx.h, count, _ptr(x), _ptr(y), count if n is None else n, C.byref(out)))
    return float(out.value)


def compare_communities(g: Graph, a, b) -> float:
    """compare_communities(g, a, b) (src/common.cpp:163-173)."""
    return nmi(g.ctx, a, b, g.n)


def truth_file_pairs(labels, path: str):
    """The confusion pairs compare_communities(g, labels, filename) builds
    (src/common.cpp:127-160): one ground-truth community per line (vertex
    ids separated by white space), numbered from 1; empty lines and lines
    starting with '#' are skipped, and a line is read as a stream of integers
    until the first character that cannot continue one (so "12abc" yields 12
    and ends the line).  Vertex ids must lie in [0, n).  Returns (community,
    labels[v]) as two int32 arrays."""
    import re

    lab = _i32(labels)
    num = re.compile(r"[+-]?\d+")
    comm, va, vb = 0, [], []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line[0] == "#":
                continue
            comm += 1
            for tok in line.split():
                mt = num.match(tok)
                if not mt:
                    break
                va.append(comm)
                vb.append(int(lab[int(mt.group())]))
                if mt.end() < len(tok):
                    break
    return np.asarray(va, np.int32), np.asarray(vb, np.int32)


def compare_communities_file(g: Graph, labels, path: str) -> float:
    """compare_communities(g, labels, filename) (src/common.cpp:127-160) on
    the device: the pairs of truth_file_pairs, normalised by g.n."""
    a, b = truth_file_pairs(labels, path)
    return nmi(g.ctx, a, b, g.n)


@dataclass
class Iteration:
    it: int
    kind: str
    score: float
    k: int
    raw: np.ndarray | None = None


@dataclass
class RunResult:
    labels: np.ndarray
    score: float
    iterations: int
    k: int
    log: list = field(default_factory=list)


THRESHOLD_ITER_CAP = 1000


def run(g: Graph, rule: Rule, strategy: int = 0, frac: float = 0.5, rounds: int = 1, n_iter: int = -1,
        threshold: float = 0.0, initial: int = 0, keep_raw: bool = False, callback=None,
        initial_on_device: bool = False) -> RunResult:
    """The reference driver loop (src/main.cpp:187-266) on the device.

    In threshold mode (n_iter == -1) the reference loops until the relative
    improvement drops to `threshold`, which never happens for a graph whose
    score stays <= 0 (e.g. a single edge); this loop, like pcd_batch_run, stops
    after THRESHOLD_ITER_CAP iterations.  `initial_on_device`: the
    triangle-based start partition (initial 1) is computed on the device
    (the same labels as the host's)."""
    rand = GlibcRand(1)
    if initial == 1 or rule.kind == 2:
        g.count_triangles()
    if initial == 0:
        g.labels = create_singleton_partition(g, rand)
    elif initial == 1 and initial_on_device:
        create_clustering_partition_device(g)
    elif initial == 1:
        g.labels = create_clustering_partition(g)
    else:
        raise ValueError("unknown partitioning strategy")
    pr = PropagationRefinement(frac)
    mr = MergingRefinement(rounds)
    prev = 0.0
    it = 0
    log = []
    while True:
        k = g.compress()
        score = rule.calculate(g)
        done = (it >= n_iter) if n_iter != -1 else (
            (prev > 0 and score > 0 and score / prev - 1 <= threshold) or it >= THRESHOLD_ITER_CAP - 1)
        if done:
            break
        if strategy == 0 or (strategy == 2 and it % 2 == 0):
            kind = "prop"
            pr.refine(g, rule, rand())
        else:
            kind = "merge"
            mr.refine(g, rule, rand())
        rec = Iteration(it, kind, score, k, g.labels if keep_raw else None)
        log.append(rec)
        if callback:
            callback(rec)
        it += 1
        prev = score
    return RunResult(g.labels, score, it, k, log)


# ---------------------------------------------------------------------------
# batched path
# ---------------------------------------------------------------------------
def pack_graphs(graphs):
    """(vertex_offsets, indices, adj) of the packed CSR of a list of
    (indices, adj) pairs: union row offsets, each graph's local neighbour ids."""
    voff = [0]
    ind_parts, adj_parts = [], []
    base = 0
    for ind, adj in graphs:
        ind = np.asarray(ind, dtype=np.int64)
        ind_parts.append(ind[:-1] + base)
        adj_parts.append(np.asarray(adj, dtype=np.int32))
        base += int(ind[-1])
        voff.append(voff[-1] + ind.shape[0] - 1)
    indices = np.concatenate(ind_parts + [np.array([base], np.int64)]).astype(np.int32)
    adj = np.concatenate(adj_parts) if adj_parts else np.zeros(0, np.int32)
    return np.asarray(voff, np.int32), indices, adj


class Batch:
    """Many graphs refined together (pcd_batch_* in include/pcd.h)."""

    def __init__(self, ctx: Context, h, voff: np.ndarray):
        self.ctx, self.h, self.voff = ctx, h, voff
        self.G = voff.shape[0] - 1
        self.n = int(voff[-1])

    @classmethod
    def from_graphs(cls, ctx: Context, graphs) -> "Batch":
        voff, indices, adj = pack_graphs(graphs)
        h = C.c_void_p()
        ctx._check(LIB.pcd_batch_load(ctx.h, voff.shape[0] - 1, _ptr(voff), _ptr(indices), _ptr(adj), C.byref(h)))
        b = cls(ctx, h, voff)
        b._hold = (indices, adj)
        return b

    @classmethod
    def from_host_ptr(cls, ctx: Context, voff: np.ndarray, indices_ptr: int, adj_ptr: int) -> "Batch":
        """Packed CSR already laid out in (pinned) host memory: union row
        offsets `indices[N+1]`, local neighbour ids `adj`."""
        voff = np.ascontiguousarray(voff, dtype=np.int32)
        h = C.c_void_p()
        ctx._check(LIB.pcd_batch_load(ctx.h, voff.shape[0] - 1, _ptr(voff), C.c_void_p(indices_ptr),
                                      C.c_void_p(adj_ptr), C.byref(h)))
        return cls(ctx, h, voff)

    def get_labels_ptr(self, host_ptr: int):
        self.ctx._check(LIB.pcd_batch_labels_get(self.h, C.c_void_p(host_ptr)))

    @classmethod
    def from_device(cls, ctx: Context, voff: np.ndarray, d_indices: int, d_adj: int) -> "Batch":
        voff = np.ascontiguousarray(voff, dtype=np.int32)
        h = C.c_void_p()
        ctx._check(LIB.pcd_batch_load_device(ctx.h, voff.shape[0] - 1, _ptr(voff), C.c_void_p(d_indices),
                                             C.c_void_p(d_adj), C.byref(h)))
        return cls(ctx, h, voff)

    def free(self):
        if self.h:
            LIB.pcd_graph_free(self.h)
            self.h = None

    @property
    def labels(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        self.ctx._check(LIB.pcd_batch_labels_get(self.h, _ptr(out)))
        return out

    @labels.setter
    def labels(self, lab):
        lab = _i32(lab)
        self.ctx._check(LIB.pcd_batch_labels_set(self.h, _ptr(lab)))

    def graph_labels(self, labels: np.ndarray, g: int) -> np.ndarray:
        return labels[self.voff[g]:self.voff[g + 1]]

    def compress(self) -> np.ndarray:
        k = np.zeros(self.G, np.int32)
        self.ctx._check(LIB.pcd_batch_compress(self.h, _ptr(k)))
        return k

    def set_bins(self, max_deg):
        arr = (C.c_int32 * 7)(*[int(x) for x in max_deg])
        self.ctx._check(LIB.pcd_graph_set_bins(self.h, arr))

    def set_hub_part(self, labels: int):
        self.ctx._check(LIB.pcd_graph_set_hub_part(self.h, int(labels)))

    def get_bins(self):
        md = (C.c_int32 * 7)()
        cnt = (C.c_int64 * 8)()
        self.ctx._check(LIB.pcd_graph_get_bins(self.h, md, cnt))
        return list(md), list(cnt)

    def stats(self):
        """Per-graph statistics: a list of (sizes, int_volume, ext_volume),
        graph g's communities numbered from 0 as in that graph alone."""
        k = self.compress()
        tot = int(k.sum())
        s = np.zeros(max(tot, 1), np.int32)
        i = np.zeros(max(tot, 1), np.int32)
        e = np.zeros(max(tot, 1), np.int32)
        self.ctx._check(LIB.pcd_stats_get(self.h, _ptr(s), _ptr(i), _ptr(e)))
        off = np.concatenate([[0], np.cumsum(k)])
        return [(s[off[g]:off[g + 1]], i[off[g]:off[g + 1]], e[off[g]:off[g + 1]]) for g in range(self.G)]

    def score(self, rule: Rule) -> np.ndarray:
        out = np.zeros(self.G, np.float64)
        self.ctx._check(LIB.pcd_batch_score(self.h, C.byref(rule._c()), _ptr(out)))
        return out

    def refine(self, rule: Rule, frac: float, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        self.ctx._check(LIB.pcd_batch_refine(self.h, C.byref(rule._c()), float(frac), _ptr(s)))

    def merge(self, rule: Rule, rounds: int, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        self.ctx._check(LIB.pcd_batch_merge(self.h, C.byref(rule._c()), int(rounds), _ptr(s)))

    def run(self, rule: Rule, strategy: int = 0, frac: float = 1.0, rounds: int = 1, n_iter: int = 10,
            threshold: float = 0.0, cuda_graph: bool = True):
        scores = np.zeros(self.G, np.float64)
        iters = np.zeros(self.G, np.int32)
        self.ctx._check(LIB.pcd_batch_run(self.h, C.byref(rule._c()), strategy, float(frac), rounds, n_iter,
                                          float(threshold), 1 if cuda_graph else 0, _ptr(scores), _ptr(iters)))
        return scores, iters


# ---------------------------------------------------------------------------
# serving loop
# ---------------------------------------------------------------------------
def estimate_device_bytes(n: int, nnz: int, max_deg: int, num_hubs: int = 0, num_graphs: int = 1,
                          iteration_cap: int = 1000, merges: bool = False, num_sms: int = 152) -> int:
    """Upper bound of the device memory a (batch) load and run needs
    (pcd_estimate_device_bytes)."""
    out = C.c_int64()
    st = LIB.pcd_estimate_device_bytes(int(n), int(nnz), int(max_deg), int(num_hubs), int(num_graphs),
                                       int(iteration_cap), 1 if merges else 0, int(num_sms), C.byref(out))
    if st:
        raise PcdError(st, "pcd_estimate_device_bytes")
    return out.value


@dataclass
class ServeResult:
    labels: np.ndarray
    score: float
    iterations: int
    latency_ms: float
    queue_ms: float
    batch_graphs: int


class Server:
    """Requests served in batches by worker threads (pcd_serve_* in
    include/pcd.h).  submit() copies the graph and returns a ticket; wait()
    blocks for that ticket's result."""

    def __init__(self, device: int = 0, workers: int = 2, max_batch_graphs: int = 256,
                 max_batch_edges: int = 1 << 28, hbm_budget_bytes: int = 150 * 10**9, max_wait_ms: float = 2.0,
                 cuda_graph: bool = False, small_graph_edges: int = 1 << 20, large_graph_edges: int = 1 << 24,
                 continuous: bool = True):
        cfg = _ServeConfig(device, workers, max_batch_graphs, max_batch_edges, hbm_budget_bytes, max_wait_ms,
                           1 if cuda_graph else 0, small_graph_edges, large_graph_edges, 1 if continuous else 0)
        self.h = C.c_void_p()
        st = LIB.pcd_serve_start(C.byref(cfg), C.byref(self.h))
        if st:
            raise PcdError(st, "pcd_serve_start")
        self._n = {}

    def submit(self, indices, adj, rule: Rule, strategy: int = 0, frac: float = 1.0, rounds: int = 1,
               n_iter: int = -1, threshold: float = 0.0) -> int:
        ind = _i32(indices)
        a = _i32(adj)
        sched = _Schedule(rule._c(), strategy, float(frac), rounds, n_iter, float(threshold))
        t = C.c_uint64()
        st = LIB.pcd_serve_submit(self.h, ind.shape[0] - 1, a.shape[0] // 2, _ptr(ind), _ptr(a), C.byref(sched),
                                  C.byref(t))
        if st:
            raise PcdError(st, "pcd_serve_submit")
        self._n[t.value] = ind.shape[0] - 1
        return t.value

    def done(self, ticket: int) -> bool:
        d = C.c_int32()
        st = LIB.pcd_serve_poll(self.h, C.c_uint64(ticket), C.byref(d))
        if st:
            raise PcdError(st, "pcd_serve_poll")
        return bool(d.value)

    def wait(self, ticket: int) -> ServeResult:
        lab = np.empty(self._n.pop(ticket), np.int32)
        score = C.c_double()
        it = C.c_int32()
        tm = _ServeTiming()
        st = LIB.pcd_serve_wait(self.h, C.c_uint64(ticket), _ptr(lab), C.byref(score), C.byref(it), C.byref(tm))
        if st:
            raise PcdError(st, f"request {ticket}")
        return ServeResult(lab, score.value, it.value, tm.latency_ms, tm.queue_ms, tm.batch_graphs)

    def stats(self) -> dict:
        out = _ServeStats()
        LIB.pcd_serve_stats_get(self.h, C.byref(out))
        return {nm: getattr(out, nm) for nm, _ in _ServeStats._fields_}

    def stop(self):
        if self.h:
            LIB.pcd_serve_stop(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()


def convert_edges(ctx: Context, edges, num_nodes: int = -1):
    """Edge list -> (Graph, map) on the device with the reference converter's
    semantics (pcd_convert_edges); map[i] is the original id of vertex i."""
    e = np.ascontiguousarray(np.asarray(edges).reshape(-1, 2), dtype=np.int32)
    src = np.ascontiguousarray(e[:, 0])
    dst = np.ascontiguousarray(e[:, 1])
    nmax = num_nodes if num_nodes >= 0 else (int(e.max()) + 1 if e.size else 0)
    mp = np.empty(max(nmax, 1), np.int32)
    h = C.c_void_p()
    ctx._check(LIB.pcd_convert_edges(ctx.h, e.shape[0], _ptr(src), _ptr(dst), int(num_nodes), _ptr(mp),
                                     C.byref(h)))
    n, m = C.c_int32(), C.c_int32()
    LIB.pcd_graph_size(h, C.byref(n), C.byref(m))
    return Graph(ctx, h, n.value, m.value), mp[: n.value].copy()
