"""A schedule run through the shim that replaces the reference's GPU host API
(cuda_init, cuda_transfer_graph, cuda_labels_to_device,
cuda_collect_statistics, cuda_propagation_step / cuda_merging_step,
cuda_labels_from_device; src/framework-cuda.cuh:14-23) gives every sweep's
labels exactly as the oracle's -p 1 schedule."""
import os
import subprocess

import numpy as np
import pytest

from conftest import golden_graph

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric,strategy", [("mod", 2), ("cpm-0.01", 0)])
def test_schedule_through_the_shim_matches_oracle(tmp_path, metric, strategy):
    import oracle
    import shim_build

    exe = os.path.join(tmp_path, "shim")
    shim_build.build(exe)
    g = golden_graph("rmat12")
    csr = os.path.join(tmp_path, "g.bin")
    with open(csr, "wb") as f:
        np.array([g.n, g.m], np.int32).tofile(f)
        g.indices.astype(np.int32).tofile(f)
        g.adj.astype(np.int32).tofile(f)
    rule, lam = oracle.parse_rule(metric)
    iters = 6
    out = os.path.join(tmp_path, "labels.bin")
    r = subprocess.run([exe, csr, out, str(rule), repr(lam), str(strategy), str(iters)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.int32).reshape(iters, g.n)
    _, _, want = oracle.run_schedule(oracle.Port(), g.indices, g.adj, metric, strategy, 1.0, 1, iters)
    assert len(want) == iters
    for k, sw in enumerate(want):
        assert np.array_equal(got[k], sw.raw), f"sweep {k} ({sw.kind})"
