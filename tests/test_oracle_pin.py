"""CPU: the oracle (our C restatement) pinned against the reference itself.

* always: the golden hashes written by the reference (tests/golden/), the
  converter's byte output, and libc's own rand()/rand_r();
* when the reference objects were built here (oracle/_ref): side-by-side runs
  of the reference and the restatement on seeded graphs.
"""
import ctypes
import hashlib

import numpy as np
import pytest

from conftest import golden_graph


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def test_generators_and_converter_bytes(golden):
    import graphs

    for name, rec in golden["graphs"].items():
        g = golden_graph(name)
        assert (g.n, g.m) == (rec["n"], rec["m"])
        assert hashlib.sha256(graphs.to_bytes(g)).hexdigest() == rec["pcd_sha256"]
        back = graphs.from_bytes(graphs.to_bytes(g))
        assert np.array_equal(back.adj, g.adj) and np.array_equal(back.indices, g.indices)


def test_format_reader_rejects_corrupt_files():
    import graphs

    g = golden_graph("rmat12")
    data = graphs.to_bytes(g)
    for bad in (b"XYZ" + data[3:], data[:-1], data + b"\0", data[:40]):
        with pytest.raises(graphs.FormatError):
            graphs.from_bytes(bad)
    # neighbour id out of range
    arr = bytearray(data)
    off = 11 + 4 * (g.n + 1)
    arr[off:off + 4] = (g.n + 5).to_bytes(4, "little")
    with pytest.raises(graphs.FormatError):
        graphs.from_bytes(bytes(arr))


def test_glibc_streams_match_libc(port):
    import oracle

    libc = ctypes.CDLL("libc.so.6")
    libc.rand.restype = ctypes.c_int
    libc.rand_r.restype = ctypes.c_int
    for seed in (1, 7, 2**31 + 5):
        libc.srand(ctypes.c_uint(seed))
        a = [libc.rand() for _ in range(5000)]
        r = oracle.GlibcRand(port.lib, seed)
        assert a == [r() for _ in range(5000)]
    s1, s2 = ctypes.c_uint(987654321), ctypes.c_uint32(987654321)
    for _ in range(20000):
        assert libc.rand_r(ctypes.byref(s1)) == port.lib.pcdo_rand_r(ctypes.byref(s2))


@pytest.mark.parametrize("idx", range(14))
def test_oracle_matches_reference_golden(port, golden, idx):
    import oracle

    case = golden["cases"][idx]
    g = golden_graph(case["graph"])
    seen = []
    oracle.run_schedule(port, g.indices, g.adj, case["metric"], case["strategy"], case["frac"], case["rounds"],
                        case["n_iter"], 0.0, case["initial"], callback=lambda sw, lab: seen.append((sw, lab.copy())))
    assert len(seen) == len(case["sweeps"])
    for (sw, lab), ref in zip(seen, case["sweeps"]):
        assert sha(lab) == ref["in_sha256"]
        assert sha(sw.raw) == ref["raw_sha256"], f"sweep {sw.it} {sw.kind}"
        assert sw.k == ref["k"]
        s, r = sw.score, float(ref["score"])
        if case["metric"] == "wcc":
            assert abs(s - r) <= 1e-12 * abs(r)  # the reference sums WCC with an OpenMP reduction
        else:
            assert s == r


def test_oracle_triangles_golden(port, golden):
    for name, rec in golden["graphs"].items():
        g = golden_graph(name)
        tri, td, cc = port.load(g.indices, g.adj).count_triangles()
        assert sha(tri) == rec["tri_sha256"] and sha(td) == rec["tri_deg_sha256"]
        assert cc == float(rec["cc"])


def test_oracle_hand_graphs(port, golden):
    import oracle

    for name, rec in golden["hand"].items():
        ind = np.array(rec["indices"], np.int32)
        adj = np.array(rec["adj"], np.int32)
        for key, case in rec["cases"].items():
            metric, s, i = key.split("/")
            final, score, sweeps = oracle.run_schedule(port, ind, adj, metric, int(s[1:]), 1.0, 1, 6, 0.0, int(i[1:]))
            assert [sw.raw.tolist() for sw in sweeps] == [x["raw"] for x in case["sweeps"]], (name, key)
            assert final.tolist() == case["final"]


needs_ref = pytest.mark.skipif("not __import__('oracle').reference_available()",
                               reason="reference objects not built here (make -C oracle ref)")


@needs_ref
@pytest.mark.parametrize("metric,strategy,frac,rounds,initial", [
    ("mod", 0, 1.0, 1, 0), ("mod", 0, 0.3, 1, 0), ("mod", 2, 1.0, 2, 0), ("cpm-0.02", 2, 1.0, 1, 0),
    ("wcc", 2, 1.0, 1, 1), ("cpm-0.2", 1, 1.0, 4, 1)])
def test_oracle_matches_reference_side_by_side(port, metric, strategy, frac, rounds, initial):
    import graphs
    import oracle

    ref = oracle.Reference("strict")
    e = graphs.rmat(11, 12, 0.55, 0.2, 0.2, seed=17)
    g = graphs.convert_edges(e)
    lr, sr, swr = oracle.run_schedule(ref, g.indices, g.adj, metric, strategy, frac, rounds, 8, 0.0, initial)
    lp, sp, swp = oracle.run_schedule(port, g.indices, g.adj, metric, strategy, frac, rounds, 8, 0.0, initial)
    assert len(swr) == len(swp)
    for a, b in zip(swr, swp):
        assert np.array_equal(a.raw, b.raw), (a.it, a.kind)
    assert abs(sr - sp) <= 1e-12 * abs(sr)


@needs_ref
def test_oracle_gains_match_reference_including_int_wrap(port):
    """Single gains, including WCC communities large enough that the
    reference's int products wrap (sizes > 46341)."""
    import graphs
    import oracle

    ref = oracle.Reference("strict")
    n = 60000
    edges = np.array([(0, i) for i in range(1, n)] + [(i, i + 1) for i in range(1, n - 1)])
    g = graphs.convert_edges(edges)
    ref.load(g.indices, g.adj)
    port.load(g.indices, g.adj)
    ref.count_triangles()
    port.count_triangles()
    lab = np.zeros(g.n, np.int32)
    lab[-5:] = 1
    for rule, lam in ((0, 0.0), (1, 0.01), (2, 0.0)):
        for (kind, a, b, k) in (("join", g.n - 1, 0, 2), ("leave", 3, 0, 2), ("leave", g.n - 2, 1, 1),
                                ("merge", 0, 1, 3), ("merge", 1, 0, 3), ("join", 5, 1, 1)):
            x = ref.gain(kind, rule, lam, lab, a, b, k)
            y = port.gain(kind, rule, lam, lab, a, b, k)
            assert (x == y) or (x != x and y != y), (rule, kind, x, y)


@needs_ref
def test_reference_shipped_flags_match_strict_except_cpm(golden):
    """The reference compiled with its Makefile flags (-ffast-math
    -march=native) against the strict-IEEE golden hashes: identical for
    Modularity and WCC; CPM differs (FMA contraction of k - lambda * size)."""
    import oracle

    ref = oracle.Reference("shipped")
    for case in golden["cases"]:
        g = golden_graph(case["graph"])
        seen = []
        oracle.run_schedule(ref, g.indices, g.adj, case["metric"], case["strategy"], case["frac"], case["rounds"],
                            case["n_iter"], 0.0, case["initial"], callback=lambda sw, lab: seen.append(sha(sw.raw)))
        same = seen == [s["raw_sha256"] for s in case["sweeps"]]
        if case["metric"].startswith("cpm"):
            continue  # contraction-dependent: fast-math may fuse k - lambda * size
        assert same, (case["graph"], case["metric"], case["strategy"])


def test_oracle_extras_golden(port, golden_extras):
    """Initial partition, connected components and NMI of the restatement
    against the reference's outputs in tests/golden/golden_extras.json."""
    import graphs
    import make_golden_extras as mge

    for name, rec in golden_extras["graphs"].items():
        g = golden_graph(name)
        if name == "forest":
            assert hashlib.sha256(graphs.to_bytes(g)).hexdigest() == golden_extras["forest_pcd_sha256"]
        port.load(g.indices, g.adj)
        port.count_triangles()
        clus = port.clustering()
        comp = port.find_connected()
        assert sha(clus) == rec["clustering_sha256"], name
        assert sha(comp) == rec["components_sha256"], name
        assert np.unique(comp).shape[0] == rec["components"]
        s1, s2 = mge.synth_labels(g.n)
        # the restatement walks the confusion map in the reference's order: bit-identical
        assert repr(port.nmi(clus, comp)) == rec["nmi_clustering_components"]
        assert repr(port.nmi(clus, s1)) == rec["nmi_clustering_synth"]
        assert repr(port.nmi(s1, s2)) == rec["nmi_synth"]
    for name, rec in golden_extras["hand"].items():
        g = graphs.convert_edges(np.array(__import__("make_golden").HAND[name]))
        port.load(g.indices, g.adj)
        port.count_triangles()
        assert port.clustering().tolist() == rec["clustering"], name
        assert port.find_connected().tolist() == rec["components"], name


def test_truth_file_pairs_match_reference_reader(port, golden_extras, tmp_path):
    """The host reader of ground-truth files (pcd.truth_file_pairs) builds the
    reference's confusion pairs: with the restatement's NMI (bit-identical to
    the reference's for the same pairs) it reproduces the value the
    reference computed from the same file (comment and empty lines
    included)."""
    import make_golden_extras as mge
    import pcd

    g = golden_graph("sbm10k")
    port.load(g.indices, g.adj)
    port.count_triangles()
    clus = port.clustering()
    path = tmp_path / "truth.txt"
    mge.truth_file(g, 100, str(path))
    a, b = pcd.truth_file_pairs(clus, str(path))
    assert a.min() == 1 and a.shape[0] == g.n
    assert repr(port.nmi(a, b, g.n)) == golden_extras["graphs"]["sbm10k"]["nmi_truth_file_clustering"]


@needs_ref
def test_truth_file_reader_edge_cases_match_reference(port, tmp_path):
    """Lines the reference's stream reader treats specially: comments, empty
    lines, a token with trailing characters (read up to them, then the line
    ends), a non-numeric token, repeated vertices, a leading '+'."""
    import graphs
    import oracle
    import pcd

    ref = oracle.Reference("strict")
    g = graphs.convert_edges(graphs.sbm(10, 30, 0.3, 0.01, seed=8))
    ref.load(g.indices, g.adj)
    port.load(g.indices, g.adj)
    rng = np.random.default_rng(3)
    labels = rng.integers(0, 7, g.n).astype(np.int32)
    text = ("# header\n\n0 1 2 3\n4 5 6x 7 8\n9 10 abc 11\n+12 13 13 14\n\n# c\n"
            + " ".join(str(v) for v in range(15, g.n)) + "\n20 21\t22\n")
    path = tmp_path / "truth.txt"
    path.write_text(text)
    a, b = pcd.truth_file_pairs(labels, str(path))
    want = ref.nmi_file(labels, str(path))
    assert repr(port.nmi(a, b, g.n)) == repr(want)


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_extras_side_by_side_with_reference(port, seed):
    """Start partition, components and NMI of the restatement against the
    reference's own objects on seeded graphs with several components."""
    import graphs
    import oracle

    ref = oracle.Reference("strict")
    rng = np.random.default_rng(seed)
    parts, off = [], 0
    for k in range(4):
        e = np.asarray(graphs.rmat(9 + k % 2, 6, 0.57, 0.19, 0.19, seed=100 * seed + k), np.int64)
        parts.append(e + off)
        off += 1 << (9 + k % 2)
    g = graphs.convert_edges(np.concatenate(parts))
    ref.load(g.indices, g.adj)
    port.load(g.indices, g.adj)
    ref.count_triangles()
    port.count_triangles()
    assert np.array_equal(port.clustering(), ref.clustering())
    comp = ref.find_connected()
    assert np.array_equal(port.find_connected(), comp)
    a = rng.integers(0, 50, g.n).astype(np.int32)
    b = (a + rng.integers(0, 3, g.n)).astype(np.int32) % 40
    for x, y in ((a, b), (a, comp), (comp, comp)):
        assert repr(port.nmi(x, y)) == repr(ref.nmi(x, y))


def test_threaded_triangles_and_wcc_score_equal_the_sequential_ones():
    """The oracle's OpenMP triangle count and WCC score (used to check the
    large power-law workload in reasonable time) give exactly the sequential
    restatement's results."""
    import numpy as np

    import graphs
    import oracle

    ind, adj, _, _ = graphs.powerlaw_torch(30000, 2.5, 8, 2000, 1.5, 20, 2000, 0.3, seed=11, device="cpu")
    p = oracle.Port().load(ind, adj)
    t1, d1, c1 = p.count_triangles()
    t4, d4, c4 = p.count_triangles(threads=4)
    assert np.array_equal(t1, t4) and np.array_equal(d1, d4) and c1 == c4
    lab, _ = p.compress(p.clustering())
    st = p.stats(lab)
    assert p.score(2, 0.0, lab, st) == p.score(2, 0.0, lab, st, threads=4)


def test_single_vertex_community_facts_behind_the_flag_word():
    """The sweep kernels replace the label of a neighbour that is alone in its
    community by that community's volume (bit 31 set) and form its gain from
    size 1, no internal edge and that volume, without reading the community's
    statistics.  Pinned here on the oracle's statistics (the reference's
    collect_statistics restated) for golden graphs under random partitions:
    such a community has internal volume 0 and external volume = volume = its
    vertex's degree, its label occurs at most once in any row, and never in
    its own vertex's row."""
    import oracle

    port = oracle.Port()
    rng = np.random.default_rng(17)
    for name in ("rmat12", "pl20k", "sbm10k"):
        g = golden_graph(name)
        port.load(g.indices, g.adj)
        deg = np.diff(g.indices)
        for k in (g.n // 2, g.n // 8, g.n // 64):
            # k random communities, and about a third of the vertices alone
            # (labels kept in [0, n), the range the reference's relabelling takes)
            lab0, k0 = port.compress(rng.integers(0, max(k, 1), size=g.n).astype(np.int32))
            alone = rng.random(g.n) < 0.33
            lab0[alone] = k0 + np.arange(int(alone.sum()), dtype=np.int32)
            comp, _ = port.compress(lab0)
            st = port.stats(comp)
            one = st.sizes == 1
            assert one.any()
            assert np.all(st.int_volume[one] == 0)
            owner = np.empty(st.k, np.int64)
            owner[comp] = np.arange(g.n)  # a single-vertex community's only vertex
            assert np.array_equal(st.ext_volume[one], deg[owner[one]])
            row_of = np.repeat(np.arange(g.n), deg)
            lab = comp[g.adj]
            flagged = one[lab]
            # at most once per row: (row, label) pairs of flagged entries are distinct
            pairs = row_of[flagged].astype(np.int64) * st.k + lab[flagged]
            assert np.unique(pairs).size == pairs.size
            # never the row's own label
            assert not np.any(lab[flagged] == comp[row_of[flagged]])
