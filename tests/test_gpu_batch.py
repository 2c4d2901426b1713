"""The batched path: every graph of a batch gets exactly the labels and the
score it gets alone through the single-graph path (and hence the reference's)."""
import numpy as np
import pytest

from conftest import golden_graph

pytestmark = pytest.mark.gpu


def _mixed_graphs():
    import graphs

    rng = np.random.default_rng(3)
    out = []
    for i, n in enumerate([200, 350, 800, 1500, 60, 3000, 900, 5000]):
        nb = max(1, n // 50)
        sizes = np.full(nb, n // nb)
        sizes[: n - sizes.sum()] += 1
        g = graphs.convert_edges(graphs.sbm_sparse(sizes, 12.0, 2.0, rng), n)
        out.append((g.indices, g.adj))
    g = golden_graph("rmat12")
    out.append((g.indices, g.adj))
    out.append((np.array([0, 1, 2], np.int32), np.array([1, 0], np.int32)))  # a single edge
    g = graphs.convert_edges(graphs.rmat(10, 8, 0.57, 0.19, 0.19, seed=5))
    out.append((g.indices, g.adj))
    return out


def _alone(ctx, ind, adj, rule, strategy, frac, rounds, n_iter, threshold=0.0):
    import pcd

    G = pcd.Graph.from_csr(ctx, ind, adj)
    res = pcd.run(G, rule, strategy, frac, rounds, n_iter, threshold, 0)
    G.free()
    return res


@pytest.mark.parametrize("metric,strategy,frac,rounds,n_iter,cuda_graph", [
    ("mod", 0, 1.0, 1, 6, True),
    ("mod", 0, 1.0, 1, 6, False),
    ("mod", 2, 1.0, 2, 8, True),
    ("cpm-0.05", 2, 1.0, 1, 6, True),
    ("mod", 0, 0.5, 1, 5, True),
    ("mod", 1, 1.0, 3, 4, False),
])
def test_batch_run_matches_each_graph_alone(ctx, metric, strategy, frac, rounds, n_iter, cuda_graph):
    import pcd

    graphs = _mixed_graphs()
    rule = pcd.parse_metric(metric)
    B = pcd.Batch.from_graphs(ctx, graphs)
    scores, iters = B.run(rule, strategy, frac, rounds, n_iter, 0.0, cuda_graph)
    labels = B.labels
    B.free()
    for i, (ind, adj) in enumerate(graphs):
        res = _alone(ctx, ind, adj, rule, strategy, frac, rounds, n_iter)
        mine = labels[B.voff[i]:B.voff[i + 1]]
        assert np.array_equal(mine, res.labels), f"graph {i}"
        assert scores[i] == res.score, f"graph {i}: {scores[i]} vs {res.score}"
        assert iters[i] == res.iterations


def test_batch_threshold_mode_stops_each_graph_on_its_own(ctx, port):
    import pcd

    # every graph here reaches a positive score (a lone edge never does: its
    # schedule would run to the iteration cap)
    graphs = [gr for gr in _mixed_graphs() if len(gr[0]) > 3]
    rule = pcd.ModularityRule()
    B = pcd.Batch.from_graphs(ctx, graphs)
    scores, iters = B.run(rule, 2, 1.0, 1, -1, 0.01, True)
    labels = B.labels
    # after the run, statistics and scores are those of every graph's final
    # labels, including graphs that left the degree classes early
    again = B.score(rule)
    stats = B.stats()
    B.free()
    for i, (ind, adj) in enumerate(graphs):
        res = _alone(ctx, ind, adj, rule, 2, 1.0, 1, -1, 0.01)
        assert iters[i] == res.iterations, f"graph {i}"
        mine = labels[B.voff[i]:B.voff[i + 1]]
        assert np.array_equal(mine, res.labels)
        assert scores[i] == res.score
        assert again[i] == res.score, f"graph {i}: score after the run"
        port.load(ind, adj)
        st = port.stats(mine)
        assert np.array_equal(stats[i][0], st.sizes), f"graph {i}: sizes after the run"
        assert np.array_equal(stats[i][1], st.int_volume), f"graph {i}: int volume after the run"
        assert np.array_equal(stats[i][2], st.ext_volume), f"graph {i}: ext volume after the run"


def test_batch_steps_after_a_run_refine_every_graph(ctx, port):
    """A run ends with every graph marked finished; single steps afterwards
    still refine every graph."""
    import oracle
    import pcd

    graphs = _mixed_graphs()[:6]
    rule = pcd.ModularityRule()
    B = pcd.Batch.from_graphs(ctx, graphs)
    B.run(rule, 0, 1.0, 1, 3, 0.0, True)
    B.compress()
    start = B.labels
    rng = np.random.default_rng(17)
    seeds = rng.integers(0, 2**31, size=B.G).astype(np.uint32)
    B.refine(rule, 1.0, seeds)
    got = B.labels
    B.labels = start
    B.merge(rule, 1, seeds)
    got_m = B.labels
    B.free()
    rk, lam = oracle.parse_rule("mod")
    moved = 0
    for i, (ind, adj) in enumerate(graphs):
        port.load(ind, adj)
        c = start[B.voff[i]:B.voff[i + 1]]
        st = port.stats(c)
        want = port.refine_prop(rk, lam, c, 1.0, seed=int(seeds[i]), st=st)
        assert np.array_equal(got[B.voff[i]:B.voff[i + 1]], want), f"graph {i}: refine after a run"
        want_m = port.refine_merge(rk, lam, c, 1, seed=int(seeds[i]), st=st)
        assert np.array_equal(got_m[B.voff[i]:B.voff[i + 1]], want_m), f"graph {i}: merge after a run"
        moved += int(np.count_nonzero(want != c))
    assert moved > 0  # the steps did change labels


def test_batch_single_steps_match_oracle(ctx, port):
    import oracle
    import pcd

    graphs = _mixed_graphs()[:5]
    B = pcd.Batch.from_graphs(ctx, graphs)
    rng = np.random.default_rng(8)
    lab = np.concatenate([rng.integers(0, max(1, (len(ind) - 1) // 7), size=len(ind) - 1) for ind, _ in graphs])
    B.labels = lab.astype(np.int32)
    k = B.compress()
    comp = B.labels
    seeds = rng.integers(0, 2**31, size=B.G).astype(np.uint32)
    for rule_s, merge in (("mod", False), ("cpm-0.1", False), ("mod", True), ("cpm-0.1", True)):
        B.labels = comp
        rule = pcd.parse_metric(rule_s)
        if merge:
            B.merge(rule, 2, seeds)
        else:
            B.refine(rule, 1.0, seeds)
        got = B.labels
        rk, lam = oracle.parse_rule(rule_s)
        for i, (ind, adj) in enumerate(graphs):
            port.load(ind, adj)
            c = comp[B.voff[i]:B.voff[i + 1]]
            st = port.stats(c)
            want = (port.refine_merge(rk, lam, c, 2, seed=int(seeds[i]), st=st) if merge
                    else port.refine_prop(rk, lam, c, 1.0, seed=int(seeds[i]), st=st))
            assert np.array_equal(got[B.voff[i]:B.voff[i + 1]], want), (rule_s, merge, i)
    assert len(k) == B.G
    B.free()
