"""The synthetic workload generators the benchmark uses (CPU)."""
import numpy as np


def _graph(voff, ind, adj, g):
    a, b = int(voff[g]), int(voff[g + 1])
    return (ind[a:b + 1] - ind[a]).astype(np.int32), adj[int(ind[a]):int(ind[b])]


def test_device_sbm_batch_has_converter_semantics():
    import graphs

    voff, ind, adj = graphs.sbm_batch_torch(count=40, median=800, device="cpu")
    ind, adj = ind.numpy(), adj.numpy()
    assert voff.shape == (41,) and ind.shape[0] == voff[-1] + 1 and ind[-1] == adj.shape[0]
    sizes = graphs.batch_sizes(40, 800, 1.2, 200, 300_000, 4)
    total_deg = 0
    for g in range(40):
        li, la = _graph(voff, ind, adj, g)
        graphs.validate(graphs.from_csr(li, la))  # symmetric, sorted rows, no loops/duplicates
        d = np.diff(li)
        assert d.min() > 0, "isolated vertices are removed"
        assert np.all(d[:-1] >= d[1:]), "vertices renumbered by decreasing degree"
        assert li.shape[0] - 1 <= sizes[g]
        total_deg += int(d.sum())
    mean_deg = total_deg / int(voff[-1])
    assert 11.0 < mean_deg < 16.0  # intra 12 + inter 2, less duplicates


def test_device_sbm_batch_is_seeded():
    import graphs

    a = graphs.sbm_batch_torch(count=8, median=400, device="cpu")
    b = graphs.sbm_batch_torch(count=8, median=400, device="cpu")
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].numpy(), b[1].numpy())
    assert np.array_equal(a[2].numpy(), b[2].numpy())


def test_pack_graphs_round_trip():
    import graphs
    import pcd

    gs = [graphs.convert_edges(graphs.sbm_sparse(np.array([30, 30, 31]), 6.0, 1.0, np.random.default_rng(s)), 91)
          for s in range(3)]
    voff, ind, adj = pcd.pack_graphs([(g.indices, g.adj) for g in gs])
    for i, g in enumerate(gs):
        li, la = _graph(voff, ind, adj, i)
        assert np.array_equal(li, g.indices) and np.array_equal(la, g.adj)
