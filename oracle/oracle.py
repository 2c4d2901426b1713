"""ctypes front-ends for the CPU oracles of the refine / merge / score path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg; never by the product.

Two back-ends with one interface:
  * `Port`       our plain-C restatement (oracle/pcd_oracle.c -> libpcd_oracle.so),
                 built on any host including the aarch64 GPU host.
  * `Reference`  the reference's own CPU objects (oracle/_ref/*/libref_capi.so,
                 built from the reference sources); available only where the
                 reference sources were present at build time.

`run_schedule` replays the reference driver's iteration loop
(src/main.cpp:226-266): compress -> statistics -> score -> stop test ->
propagation (schedule 0, or even iterations of schedule 2) or merging.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RULES = {"mod": 0, "modularity": 0, "cpm": 1, "wcc": 2}

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port() -> str:
    path = os.path.join(HERE, "libpcd_oracle.so")
    src = os.path.join(HERE, "pcd_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return path


def parse_rule(spec: str):
    """'mod' | 'wcc' | 'cpm-<lambda>' (src/main.cpp:125-141)."""
    s = spec.lower()
    if s in ("mod", "modularity"):
        return 0, 0.0
    if s == "wcc":
        return 2, 0.0
    if s.startswith("cpm-") and len(s) > 4:
        return 1, float(s[4:])
    raise ValueError(f"unknown metric: {spec}")


class _Graph(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int32), ("indices", C.c_void_p), ("adj", C.c_void_p),
                ("tri", C.c_void_p), ("tri_deg", C.c_void_p), ("clustering_coef", C.c_double)]


class _Part(C.Structure):
    _fields_ = [("num_labels", C.c_int32), ("labels", C.c_void_p), ("sizes", C.c_void_p),
                ("int_volume", C.c_void_p), ("ext_volume", C.c_void_p)]


class _Rand(C.Structure):
    _fields_ = [("r", C.c_uint32 * 34), ("pos", C.c_int32)]


@dataclass
class Stats:
    k: int
    sizes: np.ndarray
    int_volume: np.ndarray
    ext_volume: np.ndarray


class GlibcRand:
    """glibc rand() stream (restated in pcd_oracle.c), default seed 1."""

    def __init__(self, lib, seed: int = 1):
        self._lib = lib
        self._s = _Rand()
        lib.pcdo_srand(C.byref(self._s), C.c_uint32(seed))

    def __call__(self) -> int:
        return int(self._lib.pcdo_rand(C.byref(self._s)))


class Port:
    """The C restatement.  Refinement calls take the rand_r seed explicitly;
    `rand()` is the process-independent glibc stream the driver draws it from."""

    name = "port"

    def __init__(self):
        self.lib = C.CDLL(build_port())
        L = self.lib
        L.pcdo_rand.restype = C.c_int32
        L.pcdo_rand_r.restype = C.c_int32
        L.pcdo_compress_labels.restype = C.c_int32
        L.pcdo_collect_statistics.restype = C.c_int32
        for f in ("pcdo_calculate", "pcdo_calculate_mt", "pcdo_score_join", "pcdo_score_leave", "pcdo_score_merge"):
            getattr(L, f).restype = C.c_double
        L.pcdo_contract.restype = C.c_int64
        self.rand = GlibcRand(L, 1)
        self._g = None
        self._keep = []
        self.tri = None
        self.tri_deg = None
        self.cc = float("nan")

    # -- graph ------------------------------------------------------------
    def load(self, indices: np.ndarray, adj: np.ndarray):
        self.indices = np.ascontiguousarray(indices, dtype=np.int32)
        self.adj = np.ascontiguousarray(adj, dtype=np.int32)
        self.n = self.indices.shape[0] - 1
        self.m = self.adj.shape[0] // 2
        self.tri = None
        self.tri_deg = None
        self.cc = float("nan")
        self._mk_graph()
        return self

    def _mk_graph(self):
        g = _Graph()
        g.n, g.m = self.n, self.m
        g.indices = self.indices.ctypes.data
        g.adj = self.adj.ctypes.data
        g.tri = self.tri.ctypes.data if self.tri is not None else None
        g.tri_deg = self.tri_deg.ctypes.data if self.tri_deg is not None else None
        g.clustering_coef = self.cc
        self._g = g

    def srand(self, seed: int = 1):
        self.rand = GlibcRand(self.lib, seed)

    def count_triangles(self, threads: int = 1):
        """Graph::count_triangles (graph.cpp:107-175); threads > 1 runs the edge
        loop on OpenMP threads with identical results."""
        tri = np.zeros(self.n, np.int32)
        td = np.zeros(self.n, np.int32)
        cc = C.c_double()
        if threads > 1:
            self.lib.pcdo_count_triangles_mt(C.byref(self._g), tri.ctypes.data_as(C.c_void_p),
                                             td.ctypes.data_as(C.c_void_p), C.byref(cc), C.c_int32(threads))
        else:
            self.lib.pcdo_count_triangles(C.byref(self._g), tri.ctypes.data_as(C.c_void_p),
                                          td.ctypes.data_as(C.c_void_p), C.byref(cc))
        self.tri, self.tri_deg, self.cc = tri, td, cc.value
        self._mk_graph()
        return tri, td, cc.value

    # -- framework --------------------------------------------------------
    def singleton(self) -> np.ndarray:
        lab = np.zeros(self.n, np.int32)
        self.lib.pcdo_singleton_partition(C.byref(self._g), C.byref(self.rand._s),
                                          lab.ctypes.data_as(C.c_void_p))
        return lab

    def clustering(self) -> np.ndarray:
        lab = np.zeros(self.n, np.int32)
        self.lib.pcdo_clustering_partition(C.byref(self._g), lab.ctypes.data_as(C.c_void_p))
        return lab

    def find_connected(self) -> np.ndarray:
        lab = np.zeros(self.n, np.int32)
        self.lib.pcdo_find_connected(C.byref(self._g), lab.ctypes.data_as(C.c_void_p))
        return lab

    def nmi(self, a: np.ndarray, b: np.ndarray, n: int | None = None) -> float:
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        f = self.lib.pcdo_norm_mutual_info
        f.restype = C.c_double
        return float(f(C.c_int64(a.shape[0]), a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                       C.c_int32(self.n if n is None else n)))

    def compress(self, labels: np.ndarray):
        lab = np.ascontiguousarray(labels, dtype=np.int32).copy()
        k = self.lib.pcdo_compress_labels(C.c_int32(lab.shape[0]), lab.ctypes.data_as(C.c_void_p))
        return lab, int(k)

    def stats(self, labels: np.ndarray) -> Stats:
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        k = int(lab.max()) + 1 if lab.size else 0
        s = np.zeros(max(k, 1), np.int32)
        iv = np.zeros(max(k, 1), np.int32)
        ev = np.zeros(max(k, 1), np.int32)
        self.lib.pcdo_collect_statistics(C.byref(self._g), lab.ctypes.data_as(C.c_void_p),
                                         s.ctypes.data_as(C.c_void_p),
                                         iv.ctypes.data_as(C.c_void_p),
                                         ev.ctypes.data_as(C.c_void_p))
        return Stats(k, s[:k], iv[:k], ev[:k])

    def _part(self, labels, st: Stats):
        p = _Part()
        p.num_labels = st.k
        p.labels = labels.ctypes.data
        p.sizes = st.sizes.ctypes.data
        p.int_volume = st.int_volume.ctypes.data
        p.ext_volume = st.ext_volume.ctypes.data
        return p

    def score(self, rule, lam, labels, st: Stats | None = None, threads: int = 1) -> float:
        """Rule::calculate; threads > 1 runs WCC's intersections on OpenMP
        threads with an identical value."""
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        st = st or self.stats(lab)
        p = self._part(lab, st)
        if threads > 1:
            return float(self.lib.pcdo_calculate_mt(rule, C.c_double(lam), C.byref(self._g), C.byref(p),
                                                    C.c_int32(threads)))
        return float(self.lib.pcdo_calculate(rule, C.c_double(lam), C.byref(self._g), C.byref(p)))

    def gain(self, kind, rule, lam, labels, a, b, k, st: Stats | None = None) -> float:
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        st = st or self.stats(lab)
        p = self._part(lab, st)
        if kind == "join":
            return self.lib.pcdo_score_join(rule, C.c_double(lam), C.byref(self._g), C.byref(p), a, b, k)
        if kind == "leave":
            return self.lib.pcdo_score_leave(rule, C.c_double(lam), C.byref(self._g), C.byref(p), a, k)
        return self.lib.pcdo_score_merge(rule, C.c_double(lam), C.byref(self._g), C.byref(p), a, b, k)

    def refine_prop(self, rule, lam, labels, frac, seed=None, threads=1, st=None, draws=False):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        st = st or self.stats(lab)
        p = self._part(lab, st)
        if seed is None:
            seed = self.rand()
        out = np.empty(self.n, np.int32)
        d = np.zeros(self.n, np.int32) if draws else None
        self.lib.pcdo_propagation_refine(rule, C.c_double(lam), C.byref(self._g), C.byref(p),
                                         C.c_double(frac), C.c_uint32(seed), C.c_int32(threads),
                                         out.ctypes.data_as(C.c_void_p),
                                         d.ctypes.data_as(C.c_void_p) if d is not None else None)
        return (out, d) if draws else out

    def refine_merge(self, rule, lam, labels, rounds, seed=None, threads=1, st=None, partners=False):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        st = st or self.stats(lab)
        p = self._part(lab, st)
        if seed is None:
            seed = self.rand()
        out = np.empty(self.n, np.int32)
        bp = np.zeros(max(st.k, 1), np.int32)
        self.lib.pcdo_merging_refine(rule, C.c_double(lam), C.byref(self._g), C.byref(p),
                                     C.c_int32(rounds), C.c_uint32(seed), C.c_int32(threads),
                                     out.ctypes.data_as(C.c_void_p), bp.ctypes.data_as(C.c_void_p))
        return (out, bp[: st.k]) if partners else out

    def contract(self, labels, st=None):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        st = st or self.stats(lab)
        p = self._part(lab, st)
        cap = int(np.count_nonzero(lab[self.adj] != np.repeat(lab, np.diff(self.indices))))
        a = np.zeros(max(cap, 1), np.int32)
        b = np.zeros(max(cap, 1), np.int32)
        w = np.zeros(max(cap, 1), np.int32)
        np_ = self.lib.pcdo_contract(C.byref(self._g), C.byref(p), C.c_int64(cap),
                                     a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                     w.ctypes.data_as(C.c_void_p))
        return a[:np_], b[:np_], w[:np_]


class Reference:
    """The reference's own objects through oracle/ref_capi.cpp.  The
    refinement calls draw their seeds from glibc's process-wide rand(), just as
    the reference driver does."""

    name = "reference"

    def __init__(self, flavour: str = "strict"):
        path = os.path.join(HERE, "_ref", flavour, "libref_capi.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_graph_new.restype = C.c_void_p
        L.ref_graph_new.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        for f in ("ref_graph_free", "ref_count_triangles", "ref_singleton", "ref_clustering",
                  "ref_compress", "ref_stats", "ref_score", "ref_refine_prop", "ref_refine_merge",
                  "ref_gain_join", "ref_gain_leave", "ref_gain_merge"):
            getattr(L, f).argtypes = None
        L.ref_compress.restype = C.c_int
        L.ref_stats.restype = C.c_int
        L.ref_rand.restype = C.c_int
        for f in ("ref_score", "ref_gain_join", "ref_gain_leave", "ref_gain_merge"):
            getattr(L, f).restype = C.c_double
        self.h = None
        self.cc = float("nan")

    def load(self, indices, adj):
        if self.h:
            self.lib.ref_graph_free(C.c_void_p(self.h))
        self.indices = np.ascontiguousarray(indices, dtype=np.int32)
        self.adj = np.ascontiguousarray(adj, dtype=np.int32)
        self.n = self.indices.shape[0] - 1
        self.m = self.adj.shape[0] // 2
        self.h = self.lib.ref_graph_new(self.n, self.m, self.indices.ctypes.data, self.adj.ctypes.data)
        return self

    def __del__(self):
        try:
            if self.h:
                self.lib.ref_graph_free(C.c_void_p(self.h))
        except Exception:
            pass

    def srand(self, seed: int = 1):
        self.lib.ref_srand(C.c_uint(seed))

    def rand(self) -> int:
        return int(self.lib.ref_rand())

    def count_triangles(self, threads=1):
        tri = np.zeros(self.n, np.int32)
        td = np.zeros(self.n, np.int32)
        cc = C.c_double()
        self.lib.ref_count_triangles(C.c_void_p(self.h), C.c_int(threads), tri.ctypes.data_as(C.c_void_p),
                                     td.ctypes.data_as(C.c_void_p), C.byref(cc))
        self.cc = cc.value
        return tri, td, cc.value

    def singleton(self):
        lab = np.zeros(self.n, np.int32)
        self.lib.ref_singleton(C.c_void_p(self.h), lab.ctypes.data_as(C.c_void_p))
        return lab

    def clustering(self):
        lab = np.zeros(self.n, np.int32)
        self.lib.ref_clustering(C.c_void_p(self.h), lab.ctypes.data_as(C.c_void_p))
        return lab

    def find_connected(self, threads=1):
        lab = np.zeros(self.n, np.int32)
        start = np.arange(self.n, dtype=np.int32)  # the refinement ignores the partition
        self.lib.ref_find_connected(C.c_void_p(self.h), start.ctypes.data_as(C.c_void_p), C.c_int(threads),
                                    lab.ctypes.data_as(C.c_void_p))
        return lab

    def nmi_file(self, labels, path):
        lab = np.ascontiguousarray(labels, dtype=np.int32).copy()
        f = self.lib.ref_compare_file
        f.restype = C.c_double
        return float(f(C.c_void_p(self.h), lab.ctypes.data_as(C.c_void_p), str(path).encode()))

    def nmi(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.int32).copy()
        b = np.ascontiguousarray(b, dtype=np.int32).copy()
        f = self.lib.ref_compare
        f.restype = C.c_double
        return float(f(C.c_void_p(self.h), a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p)))

    def compress(self, labels):
        lab = np.ascontiguousarray(labels, dtype=np.int32).copy()
        k = self.lib.ref_compress(C.c_void_p(self.h), lab.ctypes.data_as(C.c_void_p))
        return lab, int(k)

    def stats(self, labels, threads=1) -> Stats:
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        cap = int(lab.max()) + 1 if lab.size else 1
        s = np.zeros(cap, np.int32)
        iv = np.zeros(cap, np.int32)
        ev = np.zeros(cap, np.int32)
        k = self.lib.ref_stats(C.c_void_p(self.h), lab.ctypes.data_as(C.c_void_p), C.c_int(threads),
                               s.ctypes.data_as(C.c_void_p), iv.ctypes.data_as(C.c_void_p),
                               ev.ctypes.data_as(C.c_void_p))
        return Stats(int(k), s[:k], iv[:k], ev[:k])

    def score(self, rule, lam, labels, st=None, threads=1):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        return float(self.lib.ref_score(C.c_void_p(self.h), C.c_int(rule), C.c_double(lam),
                                        lab.ctypes.data_as(C.c_void_p), C.c_int(threads)))

    def gain(self, kind, rule, lam, labels, a, b, k, st=None):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        h = C.c_void_p(self.h)
        lp = lab.ctypes.data_as(C.c_void_p)
        if kind == "join":
            return self.lib.ref_gain_join(h, C.c_int(rule), C.c_double(lam), lp, C.c_int(a), C.c_int(b), C.c_int(k))
        if kind == "leave":
            return self.lib.ref_gain_leave(h, C.c_int(rule), C.c_double(lam), lp, C.c_int(a), C.c_int(k))
        return self.lib.ref_gain_merge(h, C.c_int(rule), C.c_double(lam), lp, C.c_int(a), C.c_int(b), C.c_int(k))

    def refine_prop(self, rule, lam, labels, frac, seed=None, threads=1, st=None):
        assert seed is None, "the reference draws its own seed from rand()"
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        out = np.empty(self.n, np.int32)
        self.lib.ref_refine_prop(C.c_void_p(self.h), C.c_int(rule), C.c_double(lam),
                                 lab.ctypes.data_as(C.c_void_p), C.c_double(frac), C.c_int(threads),
                                 out.ctypes.data_as(C.c_void_p))
        return out

    def refine_merge(self, rule, lam, labels, rounds, seed=None, threads=1, st=None):
        assert seed is None
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        out = np.empty(self.n, np.int32)
        self.lib.ref_refine_merge(C.c_void_p(self.h), C.c_int(rule), C.c_double(lam),
                                  lab.ctypes.data_as(C.c_void_p), C.c_int(rounds), C.c_int(threads),
                                  out.ctypes.data_as(C.c_void_p))
        return out


def reference_available(flavour: str = "strict") -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", flavour, "libref_capi.so"))


@dataclass
class Sweep:
    it: int
    kind: str            # "prop" | "merge"
    score: float         # score of the partition the sweep started from
    k: int               # communities before the sweep
    raw: np.ndarray      # labels written by the sweep (NEW_LABEL = -1 kept)


def run_schedule(be, indices, adj, metric="mod", strategy=0, frac=1.0, rounds=1, n_iter=10,
                 threshold=0.0, initial=0, threads=1, callback=None, aux_threads=1):
    """The reference driver loop (src/main.cpp:187-266) on back-end `be`.

    `threads` is the refinements' thread count (the reference's -p: it changes
    the rand_r streams); `aux_threads` > 1 runs the port's triangle count and
    WCC score on OpenMP threads, which leaves every result unchanged.
    Returns (final compressed labels, final score, list[Sweep]).
    """
    rule, lam = parse_rule(metric)
    be.load(indices, adj)
    be.srand(1)
    aux = {"threads": aux_threads} if aux_threads > 1 and isinstance(be, Port) else {}
    if initial == 1 or rule == 2:
        be.count_triangles(**aux)
    labels = be.singleton() if initial == 0 else be.clustering()
    prev = 0.0
    it = 0
    sweeps = []
    while True:
        labels, k = be.compress(labels)
        st = be.stats(labels)
        score = be.score(rule, lam, labels, st, **aux)
        done = (it >= n_iter) if n_iter != -1 else (prev > 0 and score > 0 and score / prev - 1 <= threshold)
        if done:
            break
        if strategy == 0 or (strategy == 2 and it % 2 == 0):
            kind = "prop"
            new = be.refine_prop(rule, lam, labels, frac, threads=threads, st=st)
        else:
            kind = "merge"
            new = be.refine_merge(rule, lam, labels, rounds, threads=threads, st=st)
        sw = Sweep(it, kind, score, k, new.copy())
        sweeps.append(sw)
        if callback:
            callback(sw, labels)
        labels = new
        it += 1
        prev = score
    return labels, score, sweeps
