"""The serving loop: each request gets exactly what the graph gets alone
through the single-graph path, whatever it was batched with, and batches are
admitted only within the device-memory budget."""
import threading
import time

import numpy as np
import pytest

from conftest import golden_graph

pytestmark = pytest.mark.gpu

SCHEDULES = [  # (metric, strategy, frac, rounds, n_iter, threshold)
    ("mod", 0, 1.0, 1, 6, 0.0),
    ("cpm-0.05", 2, 1.0, 1, 6, 0.0),
    ("mod", 0, 0.5, 1, -1, 0.01),
    ("mod", 2, 1.0, 2, 8, 0.0),
]


def _graphs():
    import graphs

    rng = np.random.default_rng(12)
    out = []
    for n in [200, 350, 800, 1500, 60, 3000, 900, 5000, 420, 2600, 128, 700]:
        nb = max(1, n // 50)
        sizes = np.full(nb, n // nb)
        sizes[: n - sizes.sum()] += 1
        g = graphs.convert_edges(graphs.sbm_sparse(sizes, 12.0, 2.0, rng), n)
        out.append((g.indices, g.adj))
    g = golden_graph("rmat12")
    out.append((g.indices, g.adj))
    g = graphs.convert_edges(graphs.rmat(10, 8, 0.57, 0.19, 0.19, seed=5))
    out.append((g.indices, g.adj))
    return out


def _alone(ctx, ind, adj, sched):
    import pcd

    metric, strategy, frac, rounds, n_iter, thr = sched
    G = pcd.Graph.from_csr(ctx, ind, adj)
    res = pcd.run(G, pcd.parse_metric(metric), strategy, frac, rounds, n_iter, thr, 0)
    G.free()
    return res


@pytest.mark.parametrize("continuous", [True, False], ids=["continuous", "whole-batch"])
def test_served_results_equal_each_graph_alone(ctx, continuous):
    import pcd

    gs = _graphs()
    reqs = [(i, SCHEDULES[(i * 7 + j) % len(SCHEDULES)]) for j in range(3) for i in range(len(gs))]
    rng = np.random.default_rng(3)
    rng.shuffle(reqs)
    with pcd.Server(workers=3, max_batch_graphs=8, max_wait_ms=1.0, continuous=continuous) as srv:
        tickets = []
        # submitted from two threads at once, as a server front end would
        lock = threading.Lock()

        def submit(part):
            for i, sched in part:
                metric, strategy, frac, rounds, n_iter, thr = sched
                t = srv.submit(gs[i][0], gs[i][1], pcd.parse_metric(metric), strategy, frac, rounds, n_iter, thr)
                with lock:
                    tickets.append((t, i, sched))

        th = [threading.Thread(target=submit, args=(reqs[k::2],)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        results = [(srv.wait(t), i, sched) for t, i, sched in tickets]
        stats = srv.stats()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["batches"] < len(reqs)  # some requests shared a batch
    for res, i, sched in results:
        ref = _alone(ctx, gs[i][0], gs[i][1], sched)
        assert np.array_equal(res.labels, ref.labels), (i, sched)
        assert res.score == ref.score and res.iterations == ref.iterations, (i, sched)
        assert res.latency_ms >= res.queue_ms >= 0.0


@pytest.mark.parametrize("strategy", [0, 2])
def test_requests_join_and_leave_a_running_batch(ctx, strategy):
    """Continuous batching: requests that arrive while a batch runs join it
    between iterations, graphs whose schedule ends return while the others
    run on, and every result is the graph's result alone."""
    import pcd

    gs = _graphs()
    sched = ("mod", strategy, 1.0, 1, 60, 0.0)
    metric, _, frac, rounds, n_iter, thr = sched
    first = len(gs) - 2  # rmat12: the batch the later requests join
    order = [first] + list(range(8))
    with pcd.Server(workers=1, max_batch_graphs=16, max_wait_ms=0.0) as srv:
        tickets = []
        for k, i in enumerate(order):
            tickets.append((srv.submit(gs[i][0], gs[i][1], pcd.parse_metric(metric), strategy, frac, rounds,
                                       n_iter, thr), i))
            time.sleep(0.02 if k == 0 else 0.004)
        results = [(srv.wait(t), i) for t, i in tickets]
        st = srv.stats()
    assert st["completed"] == len(order) and st["failed"] == 0
    assert st["admitted_running"] > 0, st
    assert st["released_early"] > 0, st
    # a batch is charged what its device copy holds, returned graphs included
    # until the rebuild that drops them
    assert st["estimate_exceeded"] == 0, st
    assert 0 < st["bytes_measured_peak"] <= st["bytes_peak"], st
    for res, i in results:
        ref = _alone(ctx, gs[i][0], gs[i][1], sched)
        assert np.array_equal(res.labels, ref.labels), i
        assert res.score == ref.score and res.iterations == ref.iterations, i


def test_admission_respects_the_budget_and_rejects_oversized_requests():
    import pcd

    gs = _graphs()[:8]
    need = max(pcd.estimate_device_bytes(len(ind) - 1, len(adj), int(np.diff(ind).max()), 0, 1, 6)
               for ind, adj in gs)
    budget = int(need * 1.5)  # room for about one batch at a time
    with pcd.Server(workers=3, max_batch_graphs=4, hbm_budget_bytes=budget, max_wait_ms=0.0) as srv:
        ts = [srv.submit(ind, adj, pcd.ModularityRule(), 0, 1.0, 1, 6) for ind, adj in gs]
        for t in ts:
            srv.wait(t)
        st = srv.stats()
        assert st["completed"] == len(gs)
        assert st["bytes_peak"] <= budget
        assert st["estimate_exceeded"] == 0
        assert 0 < st["bytes_measured_peak"] <= st["bytes_peak"]
    big = golden_graph("sbm10k")
    with pcd.Server(workers=1, hbm_budget_bytes=1 << 20) as srv:  # 1 MiB holds no graph
        t = srv.submit(big.indices, big.adj, pcd.ModularityRule(), 0, 1.0, 1, 4)
        with pytest.raises(pcd.PcdError) as e:
            srv.wait(t)
        assert e.value.status == 3  # PCD_ERR_OUT_OF_MEMORY
        assert srv.stats()["failed"] == 1


def test_device_bytes_within_estimate(ctx):
    import pcd

    for name in ("sbm10k", "rmat12", "pl20k"):
        g = golden_graph(name)
        deg = np.diff(g.indices)
        for merges, strategy in ((False, 0), (True, 2)):
            B = pcd.Batch.from_graphs(ctx, [(g.indices, g.adj)])
            B.run(pcd.ModularityRule(), strategy, 1.0, 1, 6)
            held = pcd.C.c_int64()
            pcd.LIB.pcd_graph_device_bytes(B.h, pcd.C.byref(held))
            B.free()
            est = pcd.estimate_device_bytes(g.n, len(g.adj), int(deg.max()), int((deg > 8192).sum()), 1, 6, merges)
            assert 0 < held.value <= est, (name, merges, held.value, est)
