"""Generate tests/golden/golden_extras.json from the reference itself: the
initial partition, connected components and NMI rows.

Runs the reference's own CPU objects (oracle/_ref/strict/libref_capi.so,
compiled from the reference sources by `make -C oracle ref`) on the seeded
graphs of make_golden.py plus a disconnected one and the hand graphs, and
records
  * create_clustering_partition (src/framework.cpp:27-59) after
    Graph::count_triangles: SHA-256 of the labels and their count;
  * FindConnectedRefinement::refine (src/refinement.cpp:291-322): SHA-256
    and the number of components;
  * compare_communities(g, a, b) (src/common.cpp:163-173) for three pairs of
    labelings (repr of the FP64 value), and for the SBM the ground-truth file
    form (src/common.cpp:127-160) with its planted blocks.
Hand graphs store the full label arrays.

    make -C oracle ref && python tests/golden/make_golden_extras.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "par-cd_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import graphs  # noqa: E402
import oracle  # noqa: E402
from make_golden import GRAPHS, HAND, make_graph, sha  # noqa: E402


def forest_edges():
    """Disconnected: three planted-block graphs of different sizes, a path and
    a star, on disjoint id ranges."""
    parts, off = [], 0
    for i, (nb, bs) in enumerate(((10, 30), (4, 50), (20, 10))):
        e = np.asarray(graphs.sbm(n_blocks=nb, block_size=bs, p_in=0.3, p_out=0.002, seed=40 + i), np.int64)
        parts.append(e + off)
        off += nb * bs
    parts.append(np.array([(off + i, off + i + 1) for i in range(40)], np.int64))
    off += 41
    parts.append(np.array([(off, off + i) for i in range(1, 25)], np.int64))
    return np.concatenate(parts)


def synth_labels(n):
    v = np.arange(n, dtype=np.int64)
    return ((v * 7919) % 97).astype(np.int32), (v // 13).astype(np.int32)


def truth_file(g, block_size, path):
    """One planted block per line (new vertex ids), with a comment and an
    empty line that the reader skips."""
    blocks = {}
    for new, old in enumerate(g.map.tolist()):
        blocks.setdefault(old // block_size, []).append(new)
    with open(path, "w") as f:
        f.write("# planted blocks\n\n")
        for b in sorted(blocks):
            f.write(" ".join(str(x) for x in blocks[b]) + "\n")


def record(ref, g):
    ref.load(g.indices, g.adj)
    ref.count_triangles()
    clus = ref.clustering()
    comp = ref.find_connected()
    s1, s2 = synth_labels(g.n)
    return dict(n=g.n, m=g.m, clustering_sha256=sha(clus), clustering_k=int(clus.max()) + 1 if g.n else 0,
                components_sha256=sha(comp), components=int(np.unique(comp).shape[0]),
                nmi_clustering_components=repr(ref.nmi(clus, comp)), nmi_clustering_synth=repr(ref.nmi(clus, s1)),
                nmi_synth=repr(ref.nmi(s1, s2))), clus


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    ref = oracle.Reference("strict")
    out = {"graphs": {}, "hand": {}}
    for name in GRAPHS:
        _, g = make_graph(name)
        rec, clus = record(ref, g)
        if GRAPHS[name]["kind"] == "sbm":
            with tempfile.TemporaryDirectory() as td:
                path = os.path.join(td, "truth.txt")
                truth_file(g, GRAPHS[name]["args"]["block_size"], path)
                rec["nmi_truth_file_clustering"] = repr(ref.nmi_file(clus, path))
        out["graphs"][name] = rec
        print(name, rec)
    g = graphs.convert_edges(forest_edges())
    out["graphs"]["forest"] = record(ref, g)[0]
    out["forest_pcd_sha256"] = hashlib.sha256(graphs.to_bytes(g)).hexdigest()
    print("forest", out["graphs"]["forest"])
    for name, edges in HAND.items():
        g = graphs.convert_edges(np.array(edges))
        ref.load(g.indices, g.adj)
        ref.count_triangles()
        out["hand"][name] = dict(clustering=ref.clustering().tolist(), components=ref.find_connected().tolist())
    path = os.path.join(HERE, "golden_extras.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
