"""The autotuner's host side: degree-distribution signatures, the candidate
bound sets (all valid for pcd_graph_set_bins), the search and the JSON cache."""
import os

import numpy as np


def test_signature_depends_on_the_degree_shape_not_the_labels():
    import graphs
    import tune

    g = graphs.convert_edges(graphs.rmat(12, 16, 0.57, 0.19, 0.19, seed=2))
    h = graphs.convert_edges(graphs.rmat(12, 16, 0.57, 0.19, 0.19, seed=3))
    s = graphs.convert_edges(graphs.sbm(20, 50, 0.2, 0.004, seed=7))
    assert tune.signature(g.indices) == tune.signature(h.indices)  # same generator and scale
    assert tune.signature(g.indices) != tune.signature(s.indices)
    assert tune.signature(np.zeros(1, np.int32)).startswith("m2^0")


def test_candidates_are_valid_bounds():
    import tune

    caps = [4, 8, 16, 32, 256, 2048, 8192]
    cands = tune.candidate_bins()
    assert tune.DEFAULT_BINS in cands
    for b in cands:
        assert all(0 <= x <= c for x, c in zip(b, caps))
        assert all(b[i] <= b[i + 1] for i in range(6))


def test_search_keeps_the_fastest_and_installs_it(tmp_path):
    import tune

    cost = {}
    installed = []

    def apply(b, p):
        installed.append((tuple(b), p))

    def run_once():
        b, p = installed[-1]
        return cost.setdefault((b, p), 1.0 + 0.01 * (b[5] == 1024) - 0.5 * (p == 8192) - 0.2 * (b[4] == 128))

    res = tune.search(apply, run_once, reps=1)
    assert res["bins"][4] == 128 and res["bins"][5] != 1024 and res["hub_part"] == 8192
    assert installed[-1] == (tuple(res["bins"]), 8192)
    path = os.path.join(tmp_path, "t.json")
    tune.save_cache({"k": {"bins": res["bins"], "hub_part": res["hub_part"]}}, path)
    assert tune.load_cache(path)["k"]["hub_part"] == 8192
    assert tune.load_cache(os.path.join(tmp_path, "missing.json")) == {}
