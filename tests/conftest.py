"""Shared test setup: import paths, the `gpu` marker, seeded graphs and the
oracles (oracle/ is test infrastructure; only tests, smoke() and bench.py's
CPU-baseline leg use it)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
for p in (os.path.join(ROOT, "par-cd_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.Port()


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_extras():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden_extras.json")) as f:
        return json.load(f)


_GRAPHS = {}


def golden_graph(name):
    """Regenerate a golden graph from its seed (cached)."""
    if name not in _GRAPHS:
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        import graphs
        import make_golden

        if name == "forest":
            import make_golden_extras

            _GRAPHS[name] = graphs.convert_edges(make_golden_extras.forest_edges())
        else:
            _GRAPHS[name] = make_golden.make_graph(name)[1]
    return _GRAPHS[name]


@pytest.fixture(scope="session")
def ctx():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import pcd

    c = pcd.Context(0)
    yield c
    c.close()


def score_tolerance(metric, want, stats, m):
    """Largest accepted |got - want| for a Modularity / CPM score: 1e-12
    relative, or the reference's own rounding error where that is larger.
    The reference adds one FP64 term per community in sequence
    (src/rules.cpp:9-22, 121-129); that sum carries up to (k + 3) * 2^-53 *
    sum |terms| of rounding error, which dominates when the terms cancel
    (scores near zero on graphs with many communities).  The device sums are
    exact integers rounded once."""
    import oracle

    rule, lam = oracle.parse_rule(metric)
    sizes = stats.sizes.astype(np.float64)
    iv = stats.int_volume.astype(np.float64)
    ev = stats.ext_volume.astype(np.float64)
    if rule == 0:
        x = (iv + ev) / (2.0 * m)
        mag = float(np.sum(np.abs(iv / (2.0 * m)) + x * x))
    elif rule == 1:
        mag = float(np.sum(np.abs(iv) + lam * sizes * np.maximum(sizes - 1, 0))) / (2.0 * m)
    else:
        return 1e-12 * abs(want)
    k = len(sizes)
    return max(1e-12 * abs(want), (k + 3) * 2.0 ** -53 * mag)
