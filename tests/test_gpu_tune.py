"""The autotuner on the device: it times candidate degree classes and hub
part sizes on the graph, stores the winner under the graph's degree
signature, reuses it for a graph of the same shape, and the tuned
configuration gives every sweep's labels exactly as the oracle does."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tuned_configuration_is_stored_reused_and_exact(ctx, tmp_path):
    import graphs
    import oracle
    import pcd
    import tune

    ind, adj, _ = graphs.rmat_torch(17, 16, 0.57, 0.19, 0.19, seed=2, device="cuda")
    path = os.path.join(tmp_path, "tuning.json")
    rule = pcd.ModularityRule()
    G = pcd.Graph.from_csr(ctx, ind, adj)
    res = tune.tune_graph(G, rule, cache_path=path, reps=1)
    assert not res["cached"] and len(res["timings"]) >= 18
    assert res["ms"] <= res["default_ms"]
    assert G.get_bins()[0] == res["bins"]
    got = []
    pcd.run(G, rule, 2, 1.0, 1, 4, keep_raw=True, callback=got.append)
    G.free()
    _, _, want = oracle.run_schedule(oracle.Port(), ind, adj, "mod", 2, 1.0, 1, 4)
    for a, b in zip(got, want):
        assert np.array_equal(a.raw, b.raw), f"sweep {a.it} ({a.kind}) with {res['bins']}/{res['hub_part']}"
    # the same graph loaded again: taken from the cache, nothing timed
    G2 = pcd.Graph.from_csr(ctx, ind, adj)
    again = tune.tune_graph(G2, rule, cache_path=path)
    assert again["cached"] and again["bins"] == res["bins"] and again["hub_part"] == res["hub_part"]
    assert G2.get_bins()[0] == res["bins"]
    G2.free()


def test_tuned_batch_runs_equal_the_default(ctx, tmp_path):
    """A batch tuned on its first propagation step runs every graph to the
    same labels, scores and iteration counts as with the default classes."""
    import graphs
    import pcd
    import tune

    voff, d_ind, d_adj = graphs.sbm_batch_torch(64, seed=4, device="cuda")
    rule = pcd.ModularityRule()
    out = []
    for tuned in (False, True):
        B = pcd.Batch.from_device(ctx, voff, d_ind.data_ptr(), d_adj.data_ptr())
        if tuned:
            res = tune.tune_batch(B, rule, 0.5, d_ind.cpu().numpy(), cache_path=os.path.join(tmp_path, "b.json"),
                                  reps=1)
            assert B.get_bins()[0] == res["bins"]
        scores, iters = B.run(rule, 0, 0.5, 1, -1, 0.0, True)
        out.append((B.labels, scores, iters))
        B.free()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])
