"""Parity at sizes where the large-degree paths of the sweep run on real
graphs rather than planted ones: R-MAT scale 20 (rows above 8192 neighbours,
the hub class), and a graph whose largest row makes m * d exceed 2^47, the
bound of the exact integer Modularity key, so that row is re-evaluated in
FP64.  Labels bit-exact against the oracle's -p 1 schedule after every sweep."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gpu_sweeps(ctx, ind, adj, metric, strategy, n_iter):
    import pcd

    G = pcd.Graph.from_csr(ctx, ind, adj)
    got, infos = [], []

    def keep(it):
        got.append(it)
        infos.append(G.info())

    res = pcd.run(G, pcd.parse_metric(metric), strategy, 1.0, 1, n_iter, keep_raw=True, callback=keep)
    G.free()
    return got, infos, res


def _oracle_sweeps(ind, adj, metric, strategy, n_iter):
    import oracle

    return oracle.run_schedule(oracle.Port(), ind, adj, metric, strategy, 1.0, 1, n_iter)


def test_rmat_scale20_hub_rows_match_oracle(ctx):
    """R-MAT scale 20, edge factor 16 (seed 2): Modularity -s 0 and -s 2 and
    CPM(0.01) -s 2, four iterations each, against the oracle."""
    import graphs

    ind, adj, _ = graphs.rmat_torch(20, 16, 0.57, 0.19, 0.19, seed=2, device="cuda")
    deg = np.diff(ind)
    assert int((deg > 8192).sum()) > 0, "no row above 8192 neighbours: the hub class is not exercised"
    configs = [("mod", 0), ("mod", 2), ("cpm-0.01", 2)]
    mine = [_gpu_sweeps(ctx, ind, adj, m, s, 4) for m, s in configs]
    with ThreadPoolExecutor(len(configs)) as ex:
        theirs = list(ex.map(lambda c: _oracle_sweeps(ind, adj, c[0], c[1], 4), configs))
    from conftest import score_tolerance
    import oracle

    port = oracle.Port().load(ind, adj)
    m = adj.shape[0] // 2
    for (metric, strat), (got, _, res), (lab, score, want) in zip(configs, mine, theirs):
        assert len(got) == len(want)
        for a, b in zip(got, want):
            assert a.kind == b.kind
            bad = np.nonzero(a.raw != b.raw)[0]
            assert bad.size == 0, f"{metric} -s {strat} sweep {a.it} ({a.kind}): {bad.size} differ, first {bad[:6]}"
        assert np.array_equal(res.labels, lab)
        tol = score_tolerance(metric, score, port.stats(lab), m)
        assert abs(res.score - score) <= tol, f"{metric} -s {strat}: score {res.score} vs {score} (tol {tol})"


def _star_with_matching(leaves):
    """A star with `leaves` leaves whose leaves are also matched in pairs:
    m = 1.5 * leaves, and the centre's degree is `leaves`."""
    import torch

    import graphs

    c = torch.zeros(leaves, dtype=torch.int64, device="cuda")
    lv = torch.arange(1, leaves + 1, dtype=torch.int64, device="cuda")
    a = torch.arange(1, leaves, 2, dtype=torch.int64, device="cuda")
    src = torch.cat([c, a])
    dst = torch.cat([lv, a + 1])
    ind, adj, _ = graphs.csr_from_edges_torch(src, dst, leaves + 1)
    return ind, adj


def test_modularity_key_guard_rechecks_in_fp64(ctx, port):
    """m * d above 2^47: the centre's join gains are beyond the exact integer
    key's error bound, so the centre is queued and re-evaluated with the FP64
    rule (pcd_sweep_info.fallback counts it); every sweep's labels equal the
    oracle's."""
    import oracle
    import pcd

    leaves = 10_000_000
    ind, adj = _star_with_matching(leaves)
    m = adj.shape[0] // 2
    d = int(np.diff(ind).max())
    assert m * d > 2**47
    G = pcd.Graph.from_csr(ctx, ind, adj)
    port.load(ind, adj)
    lab = np.arange(G.n, dtype=np.int32)
    seeds = [1804289383, 846930886, 1681692777]
    rule = pcd.ModularityRule()
    for sweep, seed in enumerate(seeds):
        comp, _ = port.compress(lab)
        st = port.stats(comp)
        G.labels = comp
        pcd.PropagationRefinement(1.0).refine(G, rule, seed)
        info = G.info()
        want = port.refine_prop(0, 0.0, comp, 1.0, seed=seed, st=st)
        got = G.labels
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, f"sweep {sweep}: {bad.size} vertices differ, first {bad[:6]}"
        assert info.fallback >= 1, f"sweep {sweep}: the centre was not re-evaluated in FP64"
        lab = want
    G.free()


def test_concurrent_class_streams_give_the_same_labels(ctx):
    """With the degree classes on concurrent side streams (pcd_set_class_streams)
    every sweep's labels still equal the oracle's."""
    import graphs

    ind, adj, _ = graphs.rmat_torch(18, 16, 0.57, 0.19, 0.19, seed=4, device="cuda")
    ctx.class_streams(True)
    try:
        got, _, res = _gpu_sweeps(ctx, ind, adj, "mod", 2, 4)
    finally:
        ctx.class_streams(False)
    _, _, want = _oracle_sweeps(ind, adj, "mod", 2, 4)
    assert len(got) == len(want)
    for a, b in zip(got, want):
        bad = np.nonzero(a.raw != b.raw)[0]
        assert bad.size == 0, f"sweep {a.it} ({a.kind}): {bad.size} differ, first {bad[:6]}"
