"""The converter on the GPU (pcd_convert_edges, convert-cuda): the same
indices, adjacency and map as the host restatement of the reference
converter, which is pinned to the reference's own output."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _cases():
    import graphs

    rng = np.random.default_rng(7)
    out = [("random-loops-dups", rng.integers(0, 300, size=(2000, 2)), -1),
           ("gaps-and-isolated", rng.integers(0, 5000, size=(800, 2)) * 3, -1),
           ("num-nodes-given", rng.integers(0, 200, size=(600, 2)), 450),
           ("single-edge", np.array([[4, 9]]), -1),
           ("only-loops", np.array([[3, 3], [5, 5]]), -1),
           ("empty", np.zeros((0, 2), np.int64), -1),
           ("rmat12", graphs.rmat(12, 8, 0.57, 0.19, 0.19, seed=3), -1),
           ("sbm", graphs.sbm(20, 50, 0.2, 0.002, seed=1), -1)]
    e = rng.integers(0, 50_000, size=(300_000, 2))
    out.append(("large-random", e, -1))
    return out


@pytest.mark.parametrize("name,edges,num_nodes", _cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_device_converter_matches_reference_semantics(ctx, name, edges, num_nodes):
    import graphs
    import pcd

    want = graphs.convert_edges(edges, None if num_nodes < 0 else num_nodes)
    g, mp = pcd.convert_edges(ctx, edges, num_nodes)
    ind, adj = g.csr()
    assert (g.n, g.m) == (want.n, want.m)
    assert np.array_equal(ind, want.indices)
    assert np.array_equal(adj, want.adj)
    assert np.array_equal(mp, want.map)
    g.free()


def test_convert_cuda_writes_the_reference_bytes(tmp_path):
    import build
    import graphs

    build.build()
    rng = np.random.default_rng(11)
    e = rng.integers(0, 2000, size=(9000, 2))
    txt = tmp_path / "g.txt"
    txt.write_text("# a comment\n\n" + graphs.edges_to_text(e))
    out = tmp_path / "g.bin"
    r = subprocess.run([os.path.join(ROOT, "par-cd_gb300", "convert-cuda"), str(txt), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == graphs.to_bytes(graphs.convert_edges(e))
