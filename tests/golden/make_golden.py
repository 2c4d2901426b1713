"""Generate tests/golden/golden.json from the reference itself.

Runs the reference's own CPU objects (oracle/_ref/strict/libref_capi.so,
compiled from the reference sources by `make -C oracle ref`) through the
reference driver's iteration loop on seeded synthetic graphs and records, for
every sweep, the SHA-256 of the labels the sweep wrote (NEW_LABEL = -1 kept),
the number of communities and the score (repr of the FP64 value) of the
partition the sweep started from; plus triangle statistics and the contracted
edge weights of one partition.  Tiny hand-made graphs also store full label
arrays.

The graphs are regenerated from their seeds by par-cd_gb300/graphs.py; the
SHA-256 of each graph's PCD bytes is stored so a test can tell a changed
generator from a changed algorithm.  The reference converter's output for the
same edge list is checked byte-for-byte against ours here.

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "par-cd_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import graphs  # noqa: E402
import oracle  # noqa: E402

GRAPHS = {
    "sbm10k": dict(kind="sbm", args=dict(n_blocks=100, block_size=100, p_in=0.1, p_out=0.0005, seed=1)),
    "rmat12": dict(kind="rmat", args=dict(scale=12, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=2)),
    "pl20k": dict(kind="powerlaw", args=dict(n=20000, deg_exp=2.5, deg_min=8, deg_max=500, comm_exp=1.5,
                                             comm_min=20, comm_max=2000, mu=0.3, seed=3)),
}

HAND = {
    # name: undirected edge list
    "path8": [(i, i + 1) for i in range(7)],
    "star9": [(0, i) for i in range(1, 9)],
    "two_triangles_bridge": [(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (3, 5), (2, 3)],
    "two_k5_bridge": [(a, b) for a in range(5) for b in range(a + 1, 5)]
    + [(a + 5, b + 5) for a in range(5) for b in range(a + 1, 5)] + [(4, 5)],
    "ring_of_k4": sum(([(4 * c + a, 4 * c + b) for a in range(4) for b in range(a + 1, 4)]
                       + [(4 * c + 3, (4 * c + 4) % 24)] for c in range(6)), []),
    "ties_grid": [(r * 6 + c, r * 6 + c + 1) for r in range(6) for c in range(5)]
    + [(r * 6 + c, (r + 1) * 6 + c) for r in range(5) for c in range(6)],
}

CASES = [
    # graph, metric, strategy, frac, rounds, n_iter, initial
    ("sbm10k", "mod", 0, 1.0, 1, 12, 0),
    ("sbm10k", "mod", 0, 0.5, 1, 8, 0),
    ("sbm10k", "mod", 1, 1.0, 1, 8, 0),
    ("sbm10k", "mod", 2, 1.0, 1, 24, 0),
    ("sbm10k", "cpm-0.01", 0, 1.0, 1, 10, 0),
    ("sbm10k", "cpm-0.01", 2, 1.0, 1, 16, 0),
    ("sbm10k", "mod", 2, 1.0, 3, 12, 0),
    ("rmat12", "mod", 0, 1.0, 1, 10, 0),
    ("rmat12", "mod", 2, 1.0, 3, 10, 0),
    ("rmat12", "cpm-0.01", 2, 1.0, 2, 8, 1),
    ("rmat12", "wcc", 2, 1.0, 1, 6, 1),
    ("pl20k", "wcc", 0, 1.0, 1, 6, 1),
    ("pl20k", "cpm-0.01", 2, 1.0, 2, 8, 1),
    ("pl20k", "mod", 0, 0.7, 1, 6, 0),
]


def make_graph(name):
    spec = GRAPHS[name]
    edges = getattr(graphs, spec["kind"])(**spec["args"])
    return edges, graphs.convert_edges(edges)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    ref = oracle.Reference("strict")
    out = {"graphs": {}, "cases": [], "hand": {}, "contract": {}}
    conv = os.path.join(ROOT, "oracle", "_ref", "convert")
    for name in GRAPHS:
        edges, g = make_graph(name)
        data = graphs.to_bytes(g)
        with tempfile.TemporaryDirectory() as td:
            txt = os.path.join(td, "g.txt")
            binf = os.path.join(td, "g.bin")
            with open(txt, "w") as f:
                f.write(graphs.edges_to_text(edges))
            subprocess.run([conv, txt, binf], stdout=subprocess.DEVNULL, check=True)
            ref_bytes = open(binf, "rb").read()
        assert ref_bytes == data, f"converter mismatch on {name}"
        ref.load(g.indices, g.adj)
        tri, td_, cc = ref.count_triangles()
        out["graphs"][name] = dict(spec=GRAPHS[name], n=g.n, m=g.m,
                                   pcd_sha256=hashlib.sha256(data).hexdigest(),
                                   tri_sha256=sha(tri), tri_deg_sha256=sha(td_), cc=repr(cc))
        print(name, g.n, g.m)
    for gname, metric, strat, frac, rounds, n_iter, init in CASES:
        _, g = make_graph(gname)
        recs = []

        def cb(sw, labels):
            recs.append(dict(it=sw.it, kind=sw.kind, k=sw.k, score=repr(sw.score), raw_sha256=sha(sw.raw),
                             in_sha256=sha(labels)))

        final, score, sweeps = oracle.run_schedule(ref, g.indices, g.adj, metric, strat, frac, rounds, n_iter,
                                                   0.0, init, callback=cb)
        out["cases"].append(dict(graph=gname, metric=metric, strategy=strat, frac=frac, rounds=rounds,
                                 n_iter=n_iter, initial=init, sweeps=recs, final_score=repr(score),
                                 final_sha256=sha(final), final_k=int(final.max()) + 1))
        print(gname, metric, strat, frac, rounds, len(recs), score)
    # contracted weights of the sbm10k partition after 3 propagation sweeps
    _, g = make_graph("sbm10k")
    ref.load(g.indices, g.adj)
    part = {}

    def cb2(sw, labels):
        part["labels"] = labels.copy()

    oracle.run_schedule(ref, g.indices, g.adj, "mod", 0, 1.0, 1, 3, callback=cb2)
    lab = part["labels"]
    a = lab.repeat(np.diff(g.indices))
    b = lab[g.adj]
    keep = a != b
    key = a[keep].astype(np.int64) * (1 << 32) + b[keep]
    uk, cnt = np.unique(key, return_counts=True)
    out["contract"]["sbm10k_prop3"] = dict(labels_sha256=sha(lab), pairs=int(uk.shape[0]),
                                           key_sha256=hashlib.sha256(uk.astype("<i8").tobytes()).hexdigest(),
                                           w_sha256=sha(cnt.astype(np.int32)))
    for name, edges in HAND.items():
        g = graphs.convert_edges(np.array(edges))
        cases = {}
        for metric, strat, init in [("mod", 0, 0), ("mod", 2, 0), ("cpm-0.1", 2, 0), ("wcc", 2, 1), ("mod", 1, 0)]:
            seq = []

            def cb3(sw, labels):
                seq.append(dict(kind=sw.kind, raw=sw.raw.tolist(), score=repr(sw.score)))

            final, score, _ = oracle.run_schedule(ref, g.indices, g.adj, metric, strat, 1.0, 1, 6, 0.0, init,
                                                  callback=cb3)
            cases[f"{metric}/s{strat}/i{init}"] = dict(sweeps=seq, final=final.tolist(), score=repr(score))
        out["hand"][name] = dict(indices=g.indices.tolist(), adj=g.adj.tolist(), cases=cases)
    path = os.path.join(os.path.dirname(__file__), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
