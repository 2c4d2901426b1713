"""The rows next to the sweep on the GPU, against the reference's outputs
(tests/golden/golden_extras.json) and the oracle:

* pcd_clustering_partition_device == create_clustering_partition
  (src/framework.cpp:27-59), bit-exact labels;
* pcd_find_connected == FindConnectedRefinement::refine
  (src/refinement.cpp:291-322), bit-exact labels;
* pcd_nmi / pcd_nmi_device == compare_communities + norm_mutual_info
  (src/common.cpp:75-173) within 1e-12 relative, or within the reference's
  own summation error where that is larger (it adds N near-equal terms in
  sequence; the GPU adds them in a tree, and its log may differ from glibc's
  by an ulp).
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_graph

pytestmark = pytest.mark.gpu

NMI_RTOL = 1e-12


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def close(x, want, ref_err=0.0):
    """|x - want| <= 1e-12 relative, or within the reference's own summation
    error bound ref_err (nmi_scale) where that is larger."""
    want = float(want)
    if want != want:
        return x != x  # NaN where the reference's arithmetic gives NaN
    return abs(x - want) <= max(NMI_RTOL * abs(want), ref_err) or (x == want)


def nmi_scale(a, b, n):
    """Bound of the reference's own rounding: it adds its N distinct-pair
    terms one after another, so its nom carries up to N * 2^-53 * sum |term|
    of error (the sum of many near-equal terms drifts that way), while the
    GPU adds them in a tree.  Returns N * 2^-53 * 2 * sum |term| / |den|."""
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    ni = np.bincount(a).astype(np.float64)
    nj = np.bincount(b).astype(np.float64)
    key, val = np.unique(a * (int(b.max()) + 1) + b, return_counts=True)
    i, j = key // (int(b.max()) + 1), key % (int(b.max()) + 1)
    terms = val * np.log(val * float(n) / (ni[i] * nj[j]))
    den = np.sum(ni[ni > 0] * np.log(ni[ni > 0] / n)) + np.sum(nj[nj > 0] * np.log(nj[nj > 0] / n))
    return float(terms.shape[0] * 2.0**-53 * 2 * np.sum(np.abs(terms)) / abs(den))


@pytest.mark.parametrize("name", ["sbm10k", "rmat12", "pl20k", "forest"])
def test_initial_partition_components_nmi_golden(ctx, golden_extras, name):
    import make_golden_extras as mge
    import pcd

    rec = golden_extras["graphs"][name]
    g = golden_graph(name)
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    k = pcd.create_clustering_partition_device(G)
    clus = G.labels
    assert sha(clus) == rec["clustering_sha256"]
    assert k == rec["clustering_k"]
    nc = pcd.FindConnectedRefinement().refine(G)
    comp = G.labels
    assert sha(comp) == rec["components_sha256"]
    assert nc == rec["components"]
    s1, s2 = mge.synth_labels(g.n)
    assert close(pcd.compare_communities(G, clus, comp), rec["nmi_clustering_components"])
    assert close(pcd.compare_communities(G, clus, s1), rec["nmi_clustering_synth"])
    assert close(pcd.compare_communities(G, s1, s2), rec["nmi_synth"])
    if "nmi_truth_file_clustering" in rec:
        import tempfile, os

        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "truth.txt")
            mge.truth_file(g, 100, path)
            assert close(pcd.compare_communities_file(G, clus, path), rec["nmi_truth_file_clustering"])
    G.free()


def test_hand_graphs_golden(ctx, golden_extras):
    import graphs
    import make_golden
    import pcd

    for name, rec in golden_extras["hand"].items():
        g = graphs.convert_edges(np.array(make_golden.HAND[name]))
        G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
        pcd.create_clustering_partition_device(G)
        assert G.labels.tolist() == rec["clustering"], name
        pcd.FindConnectedRefinement().refine(G)
        assert G.labels.tolist() == rec["components"], name
        G.free()


@pytest.mark.parametrize("scale", [14, 16])
def test_larger_graphs_against_oracle(ctx, port, scale):
    """R-MAT graphs well past the golden sizes: labels identical to the
    restatement (pinned to the reference above), NMI within tolerance; the
    device NMI (torch tensors, no host copy) equals the host-array one."""
    import graphs
    import pcd
    import torch

    g = graphs.convert_edges(graphs.rmat(scale, 8, 0.57, 0.19, 0.19, seed=scale))
    port.load(g.indices, g.adj)
    port.count_triangles()
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    pcd.create_clustering_partition_device(G)
    clus = G.labels
    assert np.array_equal(clus, port.clustering())
    pcd.FindConnectedRefinement().refine(G)
    comp = G.labels
    assert np.array_equal(comp, port.find_connected())
    want = port.nmi(clus, comp)
    got = pcd.compare_communities(G, clus, comp)
    assert close(got, want, nmi_scale(clus, comp, g.n))
    dev = pcd.nmi(ctx, torch.from_numpy(clus).cuda(), torch.from_numpy(comp).cuda(), g.n)
    assert dev == got  # same kernels, same order
    G.free()


def test_clustering_partition_then_schedule(ctx):
    """The device initial partition feeds the WCC schedule exactly like the
    host one (run() with initial=1 uses the host restatement)."""
    import graphs
    import pcd

    g = graphs.convert_edges(graphs.rmat(11, 12, 0.55, 0.2, 0.2, seed=17))
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    host = pcd.create_clustering_partition(G)
    pcd.create_clustering_partition_device(G)
    assert np.array_equal(G.labels, host)
    G.free()


def test_nmi_edge_cases(ctx, port):
    import pcd

    # no pairs: 0/0 as in the reference
    assert np.isnan(pcd.nmi(ctx, np.zeros(0, np.int32), np.zeros(0, np.int32), 5))
    # identical labelings: 1 up to rounding
    a = np.random.default_rng(1).integers(0, 50, 10_000).astype(np.int32)
    assert abs(pcd.nmi(ctx, a, a) - 1.0) < 1e-12
    # single community each side: -0/0 in the reference (NaN)
    z = np.zeros(100, np.int32)
    assert np.isnan(pcd.nmi(ctx, z, z)) and np.isnan(port.nmi(z, z, 100))
    # sparse label ids (gaps), one pair repeated
    b = (a * 1000 + 7).astype(np.int32)
    assert close(pcd.nmi(ctx, a, b), port.nmi(a, b, a.shape[0]))
    # a product ni * nj past 2^31 wraps in the reference's int arithmetic
    big = np.zeros(70_000, np.int32)
    other = np.zeros(70_000, np.int32)
    other[:5] = 1
    assert close(pcd.nmi(ctx, big, other), port.nmi(big, other, 70_000))
    with pytest.raises(pcd.PcdError):
        pcd.nmi(ctx, np.array([0, -1], np.int32), np.array([0, 0], np.int32))


def test_components_edge_cases(ctx):
    import graphs
    import pcd

    # one edge; then many tiny components
    g = graphs.convert_edges(np.array([[0, 1]]))
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    assert pcd.FindConnectedRefinement().refine(G) == 1
    assert G.labels.tolist() == [0, 0]
    G.free()
    e = np.array([(2 * i, 2 * i + 1) for i in range(5000)])
    g = graphs.convert_edges(e)
    G = pcd.Graph.from_csr(ctx, g.indices, g.adj)
    assert pcd.FindConnectedRefinement().refine(G) == 5000
    lab = G.labels
    want = np.minimum(np.arange(g.n), [g.adj[g.indices[v]] for v in range(g.n)])
    assert np.array_equal(lab, want)
    G.free()
