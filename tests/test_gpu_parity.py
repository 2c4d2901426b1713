"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own golden hashes: labels bit-exact after every sweep, integer
statistics and contracted weights exact, FP64 scores within 1e-12 relative."""
import hashlib

import numpy as np
import pytest

from conftest import golden_graph

pytestmark = pytest.mark.gpu

REL = 1e-12


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def close(a, b, rel=REL):
    return a == b or abs(a - b) <= rel * max(abs(a), abs(b))


def gpu_schedule(ctx, indices, adj, metric, strategy, frac, rounds, n_iter, initial):
    import pcd

    g = pcd.Graph.from_csr(ctx, indices, adj)
    recs = []
    res = pcd.run(g, pcd.parse_metric(metric), strategy, frac, rounds, n_iter, 0.0, initial, keep_raw=True,
                  callback=recs.append)
    out = (recs, res, g.info())
    g.free()
    return out


def oracle_schedule(port, indices, adj, metric, strategy, frac, rounds, n_iter, initial):
    import oracle

    return oracle.run_schedule(port, indices, adj, metric, strategy, frac, rounds, n_iter, 0.0, initial)


CASES = [
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


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(map(str, c)))
def test_schedule_matches_reference_golden(ctx, golden, case):
    gname, metric, strat, frac, rounds, n_iter, init = case
    g = golden_graph(gname)
    ref = next(c for c in golden["cases"]
               if (c["graph"], c["metric"], c["strategy"], c["frac"], c["rounds"], c["n_iter"], c["initial"]) == case)
    recs, res, _ = gpu_schedule(ctx, g.indices, g.adj, metric, strat, frac, rounds, n_iter, init)
    assert len(recs) == len(ref["sweeps"])
    for mine, theirs in zip(recs, ref["sweeps"]):
        assert mine.kind == theirs["kind"]
        assert mine.k == theirs["k"], f"sweep {mine.it}: communities"
        assert close(mine.score, float(theirs["score"])), f"sweep {mine.it}: score {mine.score} vs {theirs['score']}"
        assert sha(mine.raw) == theirs["raw_sha256"], f"sweep {mine.it} ({mine.kind}): labels differ"
    assert sha(res.labels) == ref["final_sha256"]
    assert close(res.score, float(ref["final_score"]))


@pytest.mark.parametrize("case", CASES[:4] + CASES[7:9] + CASES[11:], ids=lambda c: "-".join(map(str, c)))
def test_schedule_matches_oracle_arrays(ctx, port, case):
    """Same schedule against the oracle port, comparing whole arrays (a failure
    shows which vertices differ)."""
    gname, metric, strat, frac, rounds, n_iter, init = case
    g = golden_graph(gname)
    recs, res, _ = gpu_schedule(ctx, g.indices, g.adj, metric, strat, frac, rounds, n_iter, init)
    _, _, sweeps = oracle_schedule(port, g.indices, g.adj, metric, strat, frac, rounds, n_iter, init)
    for mine, theirs in zip(recs, sweeps):
        bad = np.nonzero(mine.raw != theirs.raw)[0]
        assert bad.size == 0, f"sweep {mine.it} {mine.kind}: {bad.size} vertices differ, first {bad[:8]}"


def test_stats_and_triangles_exact(ctx, port, golden):
    import pcd

    for name in ("sbm10k", "rmat12", "pl20k"):
        g = golden_graph(name)
        G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
        tri, td, cc = G.count_triangles()
        assert sha(tri) == golden["graphs"][name]["tri_sha256"]
        assert sha(td) == golden["graphs"][name]["tri_deg_sha256"]
        assert cc == float(golden["graphs"][name]["cc"])  # bit-exact: summed in vertex order
        rng = np.random.default_rng(5)
        lab = rng.integers(0, max(1, g.n // 20), size=g.n).astype(np.int32)
        lab[rng.random(g.n) < 0.05] = -1
        G.labels = lab
        k = G.compress()
        comp, k2 = port.load(g.indices, g.adj).compress(lab)
        assert k == k2
        assert np.array_equal(G.labels, comp)
        s, i, e = G.stats()
        st = port.stats(comp)
        assert np.array_equal(s, st.sizes) and np.array_equal(i, st.int_volume) and np.array_equal(e, st.ext_volume)
        G.free()


def test_contracted_weights_exact(ctx, port, golden):
    import oracle
    import pcd

    g = golden_graph("sbm10k")
    part = {}
    oracle.run_schedule(port, g.indices, g.adj, "mod", 0, 1.0, 1, 3, callback=lambda sw, lab: part.update(l=lab.copy()))
    lab = part["l"]
    assert sha(lab) == golden["contract"]["sbm10k_prop3"]["labels_sha256"]
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    G.labels = lab
    a, b, w = G.contract()
    pa, pb, pw = port.contract(lab)
    assert np.array_equal(a, pa) and np.array_equal(b, pb) and np.array_equal(w, pw)
    key = a.astype(np.int64) * (1 << 32) + b
    assert a.shape[0] == golden["contract"]["sbm10k_prop3"]["pairs"]
    assert hashlib.sha256(key.astype("<i8").tobytes()).hexdigest() == golden["contract"]["sbm10k_prop3"]["key_sha256"]
    assert sha(w) == golden["contract"]["sbm10k_prop3"]["w_sha256"]
    G.free()


def test_hand_graphs(ctx, golden):
    import pcd

    for name, rec in golden["hand"].items():
        ind = np.array(rec["indices"], np.int32)
        adj = np.array(rec["adj"], np.int32)
        for key, case in rec["cases"].items():
            metric, s, i = key.split("/")
            recs, res, _ = gpu_schedule(ctx, ind, adj, metric, int(s[1:]), 1.0, 1, 6, int(i[1:]))
            for mine, theirs in zip(recs, case["sweeps"]):
                assert mine.raw.tolist() == theirs["raw"], f"{name} {key} sweep {mine.it}"
            assert res.labels.tolist() == case["final"], f"{name} {key}"
            assert close(res.score, float(case["score"])), f"{name} {key}"


def test_single_sweeps_many_seeds(ctx, port):
    """One propagation and one merge sweep from a mid-run partition, many seeds."""
    import pcd

    g = golden_graph("rmat12")
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    port.load(g.indices, g.adj)
    rng = np.random.default_rng(11)
    for trial in range(6):
        lab = rng.integers(0, 60 + 40 * trial, size=g.n).astype(np.int32)
        comp, _ = port.compress(lab)
        st = port.stats(comp)
        for rule_s in ("mod", "cpm-0.05"):
            rule = pcd.parse_metric(rule_s)
            import oracle

            rk, lam = oracle.parse_rule(rule_s)
            seed = int(rng.integers(0, 2**31))
            G.labels = comp
            pcd.PropagationRefinement(1.0).refine(G, rule, seed)
            mine = G.labels
            theirs = port.refine_prop(rk, lam, comp, 1.0, seed=seed, st=st)
            assert np.array_equal(mine, theirs), (trial, rule_s, "prop")
            G.labels = comp
            pcd.MergingRefinement(1 + trial % 3).refine(G, rule, seed)
            mine = G.labels
            theirs = port.refine_merge(rk, lam, comp, 1 + trial % 3, seed=seed, st=st)
            assert np.array_equal(mine, theirs), (trial, rule_s, "merge")
    G.free()


def test_edge_cases(ctx, port):
    import pcd

    # empty graph
    G = pcd.Graph.from_csr(ctx, np.zeros(1, np.int32), np.zeros(0, np.int32))
    assert G.compress() == 0
    pcd.PropagationRefinement(1.0).refine(G, pcd.ModularityRule(), 1)
    G.free()
    # isolated vertices inside the vertex range, a star, a single edge
    ind = np.array([0, 3, 3, 4, 5, 6, 6], np.int32)
    adj = np.array([2, 3, 4, 0, 0, 0], np.int32)
    for metric in ("mod", "cpm-0.5"):
        recs, res, _ = gpu_schedule(ctx, ind, adj, metric, 2, 1.0, 1, 6, 0)
        _, _, sweeps = oracle_schedule(port, ind, adj, metric, 2, 1.0, 1, 6, 0)
        for a, b in zip(recs, sweeps):
            assert np.array_equal(a.raw, b.raw)
    # invalid CSR is rejected
    with pytest.raises(pcd.PcdError):
        pcd.Graph.from_csr(ctx, np.array([0, 1, 2], np.int32), np.array([1, 1], np.int32))  # loop 1-1
    with pytest.raises(pcd.PcdError):
        pcd.Graph.from_csr(ctx, np.array([0, 2, 2], np.int32), np.array([1, 1], np.int32))  # duplicate
    with pytest.raises(pcd.PcdError):
        pcd.Graph.from_csr(ctx, np.array([0, 1, 2], np.int32), np.array([1, 5], np.int32))  # out of range
    with pytest.raises(pcd.PcdError):
        pcd.Graph.from_csr(ctx, np.array([0, 3, 2, 4], np.int32), np.array([1, 2, 3, 0], np.int32))  # offsets fall
    with pytest.raises(pcd.PcdError):
        pcd.Graph.from_csr(ctx, np.array([0, 1, 2, 2], np.int32), np.array([1, 0, 2, 1], np.int32))  # span < 2m
    # rows longer than 16 neighbours are checked by a whole warp: a star of 20
    # leaves whose centre row carries one fault at a time
    leaves = np.arange(1, 21, dtype=np.int32)
    ind_star = np.concatenate([[0, 20], 20 + np.arange(1, 21)]).astype(np.int32)
    for centre, what in ((np.r_[leaves[:4], leaves[3], leaves[5:]], "duplicate"),
                         (np.r_[leaves[:10], 0, leaves[11:]], "loop"),
                         (np.r_[leaves[:10], 25, leaves[11:]], "out of range"),
                         (np.r_[leaves[10:], leaves[:10]], "unsorted")):
        adj_star = np.concatenate([centre, np.zeros(20, np.int32)]).astype(np.int32)
        with pytest.raises(pcd.PcdError, match="not a valid CSR"):
            pcd.Graph.from_csr(ctx, ind_star, adj_star)  # the centre row has a `what`
    G = pcd.Graph.from_csr(ctx, ind_star, np.concatenate([leaves, np.zeros(20, np.int32)]).astype(np.int32))
    assert G.n == 21
    G.free()
    G = pcd.Graph.from_csr(ctx, np.array([0, 1, 2], np.int32), np.array([1, 0], np.int32))
    with pytest.raises(pcd.PcdError):
        G.labels = np.array([0, 7], np.int32)
    with pytest.raises(pcd.PcdError):
        pcd.PropagationRefinement(0.0).refine(G, pcd.ModularityRule(), 1)
    with pytest.raises(pcd.PcdError):
        pcd.MergingRefinement(0).refine(G, pcd.ModularityRule(), 1)
    G.free()


BIN_LAYOUTS = [
    [4, 8, 16, 32, 256, 2048, 8192],   # default
    [0, 0, 0, 0, 0, 0, 0],             # everything in the hub class (parts over per-block slices)
    [0, 0, 0, 0, 0, 0, 8192],          # everything in 1024-thread shared-table blocks
    [0, 0, 0, 0, 0, 2048, 2048],       # 256-thread blocks (+ HBM beyond)
    [0, 0, 0, 0, 256, 256, 256],       # warps (+ HBM beyond)
    [4, 4, 4, 4, 4, 4, 4],             # 4-lane groups, the rest in HBM
    [2, 5, 9, 20, 60, 200, 700],       # a bit of everything
]


@pytest.mark.parametrize("bins", BIN_LAYOUTS, ids=lambda b: "-".join(map(str, b)))
@pytest.mark.parametrize("gname,metric", [("rmat12", "mod"), ("pl20k", "cpm-0.01"), ("rmat12", "wcc")])
def test_every_kernel_class_matches_oracle(ctx, port, bins, gname, metric):
    """The same sweeps with vertices forced into each kernel class."""
    import oracle
    import pcd

    g = golden_graph(gname)
    init = 1 if metric == "wcc" else 0
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    G.set_bins(bins)
    got = []
    pcd.run(G, pcd.parse_metric(metric), 0, 1.0, 1, 4, 0.0, init, keep_raw=True, callback=got.append)
    G.free()
    _, _, want = oracle.run_schedule(port, g.indices, g.adj, metric, 0, 1.0, 1, 4, 0.0, init)
    for a, b in zip(got, want):
        bad = np.nonzero(a.raw != b.raw)[0]
        assert bad.size == 0, f"sweep {a.it}: {bad.size} vertices differ, first {bad[:6]}"


@pytest.mark.parametrize("bins", BIN_LAYOUTS, ids=lambda b: "-".join(map(str, b)))
def test_singleton_partitions_match_oracle(ctx, port, bins):
    """Partitions of single vertices (k = n after compress) take the sweep
    path without histograms and the statistics without neighbour reads.
    Besides the start of every schedule they arise from any labeling with
    all labels distinct: a permutation of the ids, NEW_LABEL everywhere.
    Propagation (frac 1.0 and 0.6) and merge sweeps, every rule (WCC from
    singletons too), vertices forced into each kernel class, against the
    oracle."""
    import oracle
    import pcd

    g = golden_graph("rmat12")
    port.load(g.indices, g.adj)
    port.count_triangles()
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    G.set_bins(bins)
    rng = np.random.default_rng(23)
    starts = {"permutation": rng.permutation(g.n).astype(np.int32), "new labels": np.full(g.n, -1, np.int32)}
    for metric in ("mod", "cpm-0.01", "wcc"):
        rule = pcd.parse_metric(metric)
        rk, lam = oracle.parse_rule(metric)
        for name, lab in starts.items():
            comp, k = port.compress(lab)
            assert k == g.n
            st = port.stats(comp)
            G.labels = lab
            assert G.compress() == g.n
            s, i, e = G.stats()
            assert np.array_equal(s, st.sizes) and np.array_equal(i, st.int_volume) and np.array_equal(e, st.ext_volume)
            for frac in (1.0, 0.6):
                seed = int(rng.integers(0, 2**31))
                G.labels = lab
                pcd.PropagationRefinement(frac).refine(G, rule, seed)
                want = port.refine_prop(rk, lam, comp, frac, seed=seed, st=st)
                bad = np.nonzero(G.labels != want)[0]
                assert bad.size == 0, f"{metric} {name} frac {frac}: {bad.size} differ, first {bad[:6]}"
            seed = int(rng.integers(0, 2**31))
            G.labels = lab
            pcd.MergingRefinement(1).refine(G, rule, seed)
            assert np.array_equal(G.labels, port.refine_merge(rk, lam, comp, 1, seed=seed, st=st)), (metric, name)
    G.free()


def test_larger_rmat_sweeps_match_oracle(ctx, port):
    """R-MAT scale 16 (hubs above 8192 neighbours only appear at larger
    scales; the layouts above cover that class on small graphs)."""
    import graphs
    import oracle
    import pcd

    g = graphs.convert_edges(graphs.rmat(16, 16, 0.57, 0.19, 0.19, seed=9))
    for metric, strat in (("mod", 0), ("mod", 2), ("cpm-0.02", 2)):
        G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
        got = []
        pcd.run(G, pcd.parse_metric(metric), strat, 1.0, 1, 4, keep_raw=True, callback=got.append)
        G.free()
        _, _, want = oracle.run_schedule(port, g.indices, g.adj, metric, strat, 1.0, 1, 4)
        for a, b in zip(got, want):
            bad = np.nonzero(a.raw != b.raw)[0]
            assert bad.size == 0, f"{metric} s{strat} sweep {a.it}: {bad.size} differ"


def _regular_bipartite(a, b):
    """K_{a,b}: every vertex on a side has the same degree, so equal integer
    keys from different (count, volume) pairs are common."""
    rows = [[a + j for j in range(b)] for _ in range(a)] + [[i for i in range(a)] for _ in range(b)]
    ind = np.zeros(a + b + 1, np.int32)
    ind[1:] = np.cumsum([len(r) for r in rows])
    return ind, np.concatenate(rows).astype(np.int32)


def _ring_lattice(n, k):
    rows = [sorted({(v + s) % n for s in range(-k, k + 1) if s}) for v in range(n)]
    ind = np.zeros(n + 1, np.int32)
    ind[1:] = np.cumsum([len(r) for r in rows])
    return ind, np.concatenate(rows).astype(np.int32)


@pytest.mark.parametrize("shape", ["ring-60-3", "ring-400-10", "kab-40-60", "kab-300-320"])
def test_fp64_recheck_lists_match_oracle(ctx, port, shape):
    """Modularity sweeps whose integer keys tie across different (count,
    volume) pairs or equal the leave key: those vertices are re-evaluated in
    FP64, one warp per vertex up to degree 256 and one block per vertex above
    (kab-300-320 has degrees 300 and 320 only)."""
    import pcd

    kind, x, y = shape.split("-")
    ind, adj = _ring_lattice(int(x), int(y)) if kind == "ring" else _regular_bipartite(int(x), int(y))
    n = ind.shape[0] - 1
    G = pcd.Graph.from_csr(ctx, ind, adj)
    port.load(ind, adj)
    rng = np.random.default_rng(21)
    rechecked = 0
    for trial in range(8):
        lab = rng.integers(0, max(2, n // (2 + trial)), size=n).astype(np.int32)
        comp, _ = port.compress(lab)
        st = port.stats(comp)
        seed = int(rng.integers(0, 2**31))
        G.labels = comp
        pcd.PropagationRefinement(1.0).refine(G, pcd.ModularityRule(), seed)
        rechecked += G.info().fallback
        theirs = port.refine_prop(0, 0.0, comp, 1.0, seed=seed, st=st)
        bad = np.nonzero(G.labels != theirs)[0]
        assert bad.size == 0, f"trial {trial}: {bad.size} vertices differ, first {bad[:6]}"
    G.free()
    assert rechecked > 0, "no vertex took the FP64 re-evaluation path"


def _planted_degree_graph(D, hubs=8, seed=0):
    """Random base graph (average degree ~10) plus `hubs` vertices with exactly
    D neighbours each, so the degree sub-range holding D has largest degree D
    and the kernel variant sized for it runs."""
    import graphs

    n = max(6000, 2 * D)
    rng = np.random.default_rng(seed + D)
    base = rng.integers(0, n, size=(5 * n, 2))
    extra = [(n + h, int(u)) for h in range(hubs) for u in rng.choice(n, size=D, replace=False)]
    return graphs.convert_edges(np.concatenate([base, np.array(extra)]))


@pytest.mark.parametrize("D", [600, 900, 1200, 1800, 2300, 2900, 3500, 5000, 9000])
def test_block_variants_by_degree_match_oracle(ctx, port, D):
    """Each shared-table variant (positions per lane fitted to the sub-range's
    largest degree) and the hub kernel, on graphs whose largest degrees are
    planted: Modularity and CPM sweeps against the oracle."""
    import oracle
    import pcd

    g = _planted_degree_graph(D)
    assert int(np.diff(g.indices).max()) == D
    for metric in ("mod", "cpm-0.05"):
        G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
        got = []
        pcd.run(G, pcd.parse_metric(metric), 0, 1.0, 1, 4, keep_raw=True, callback=got.append)
        G.free()
        _, _, want = oracle.run_schedule(port, g.indices, g.adj, metric, 0, 1.0, 1, 4)
        for a, b in zip(got, want):
            bad = np.nonzero(a.raw != b.raw)[0]
            assert bad.size == 0, f"D={D} {metric} sweep {a.it}: {bad.size} differ"


def test_hub_label_count_past_key_width_matches_oracle(ctx, port):
    """A hub whose row holds one community 20,000 times (more than the 14 bits
    the packed integer Modularity key keeps for a count) beside 500 single-vertex
    communities: the hub is decided in FP64, and every label of the sweep equals
    the oracle's, for Modularity and CPM."""
    import graphs
    import oracle
    import pcd

    A, S = 20000, 500
    hub_edges = [(0, u) for u in range(1, A + S + 1)]
    ring = [(u, u + 1) for u in range(1, A)]
    rng = np.random.default_rng(5)
    tail = rng.integers(A + 1, A + S + 1, size=(2 * S, 2))
    g = graphs.convert_edges(np.concatenate([np.array(hub_edges + ring), tail]))
    assert int(np.diff(g.indices).max()) >= A + S
    lab = np.arange(g.n, dtype=np.int32)
    # the converter renumbers vertices: find the hub by its degree, and put
    # its neighbours of degree 3 (the ring's interior, with a few tail
    # vertices) in one community
    deg = np.diff(g.indices)
    hub = int(np.argmax(deg))
    nbr = g.adj[g.indices[hub]:g.indices[hub + 1]]
    three = nbr[deg[nbr] == 3]
    assert three.size > 0x3FFF
    lab[three] = lab[three[0]]
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    port.load(g.indices, g.adj)
    comp, _ = port.compress(lab)
    st = port.stats(comp)
    assert int(np.bincount(comp)[comp[hub]]) == 1
    for rule_s in ("mod", "cpm-0.0001"):
        rk, lam = oracle.parse_rule(rule_s)
        for seed in (3, 77):
            G.labels = comp
            pcd.PropagationRefinement(1.0).refine(G, pcd.parse_metric(rule_s), seed)
            mine = G.labels
            theirs = port.refine_prop(rk, lam, comp, 1.0, seed=seed, st=st)
            assert np.array_equal(mine, theirs), (rule_s, seed, int(np.sum(mine != theirs)))
    G.free()


@pytest.mark.parametrize("part", [1024, 8192])
def test_hub_parts_match_oracle(ctx, port, part):
    """Every row above 32 neighbours in the hub class, its other-than-single
    entries split into parts of at most `part` (several parts on the planted
    9,000-neighbour rows at 1,024, one part at 8,192): Modularity and CPM
    sweeps against the oracle."""
    import oracle
    import pcd

    g = _planted_degree_graph(9000)
    for metric in ("mod", "cpm-0.05"):
        G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
        G.set_bins([4, 8, 16, 32, 32, 32, 32])
        G.set_hub_part(part)
        got = []
        pcd.run(G, pcd.parse_metric(metric), 0, 1.0, 1, 4, keep_raw=True, callback=got.append)
        G.free()
        _, _, want = oracle.run_schedule(port, g.indices, g.adj, metric, 0, 1.0, 1, 4)
        for a, b in zip(got, want):
            bad = np.nonzero(a.raw != b.raw)[0]
            assert bad.size == 0, f"part {part} {metric} sweep {a.it}: {bad.size} differ"
