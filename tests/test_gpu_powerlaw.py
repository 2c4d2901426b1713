"""The power-law planted-community workload at a reduced size (500 000
vertices, degrees up to 5 000): CPM(0.01) from singletons and WCC from the
triangle-based start partition, each through the -s 2 schedule, against the
oracle's -p 1 schedule: every sweep's labels bit-exact, the triangle counts
and the contracted weights (a, b, w) exact, scores within 1e-12 (or the
reference's own summation bound)."""
import os

import numpy as np
import pytest

from conftest import score_tolerance

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plgraph():
    import graphs

    ind, adj, _, _ = graphs.powerlaw_torch(500_000, 2.5, 8, 5000, 1.5, 20, 20000, 0.3, seed=3, device="cuda")
    return ind, adj


@pytest.mark.parametrize("metric,init", [("cpm-0.01", 0), ("wcc", 1)])
def test_powerlaw_schedule_matches_oracle(ctx, plgraph, metric, init):
    import oracle
    import pcd

    ind, adj = plgraph
    m = adj.shape[0] // 2
    assert int(np.diff(ind).max()) > 2048  # the block and large-block classes run
    G = pcd.Graph.from_csr(ctx, ind, adj)
    res = pcd.run(G, pcd.parse_metric(metric), 2, 1.0, 1, 4, 0.0, init, keep_raw=True, initial_on_device=True)
    a, b, w = G.contract()
    tri, td, cc = G.count_triangles() if init == 1 else (None, None, None)
    G.free()
    port = oracle.Port()
    lab, score, sweeps = oracle.run_schedule(port, ind, adj, metric, 2, 1.0, 1, 4, 0.0, init,
                                             aux_threads=max(1, (os.cpu_count() or 2) - 1))
    assert len(res.log) == len(sweeps)
    for x, y in zip(res.log, sweeps):
        assert x.kind == y.kind
        bad = np.nonzero(x.raw != y.raw)[0]
        assert bad.size == 0, f"{metric} sweep {x.it} ({x.kind}): {bad.size} differ, first {bad[:6]}"
    assert np.array_equal(res.labels, lab)
    if init == 1:
        assert np.array_equal(tri, port.tri) and np.array_equal(td, port.tri_deg) and cc == port.cc
    st = port.stats(lab)
    pa, pb, pw = port.contract(lab, st)
    assert np.array_equal(a, pa) and np.array_equal(b, pb) and np.array_equal(w, pw)
    tol = score_tolerance(metric, score, st, m)
    assert abs(res.score - score) <= tol, f"{metric}: {res.score} vs {score}"
