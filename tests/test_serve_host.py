"""Host-side pieces of the serving loop (no GPU): the admission estimate and
argument checks."""
import pytest


def test_estimate_grows_with_every_input():
    import pcd

    base = pcd.estimate_device_bytes(10_000, 140_000, 40, 0, 1, 10, False, 152)
    assert base > 4 * 10_000 + 8 * 140_000  # at least the CSR and the tie slots
    assert pcd.estimate_device_bytes(20_000, 140_000, 40, 0, 1, 10, False, 152) > base
    assert pcd.estimate_device_bytes(10_000, 280_000, 40, 0, 1, 10, False, 152) > base
    assert pcd.estimate_device_bytes(10_000, 140_000, 4000, 0, 1, 10, False, 152) > base
    assert pcd.estimate_device_bytes(10_000, 140_000, 40, 3, 1, 10, False, 152) > base
    assert pcd.estimate_device_bytes(10_000, 140_000, 40, 0, 64, 1000, False, 152) > base
    assert pcd.estimate_device_bytes(10_000, 140_000, 40, 0, 1, 10, True, 152) > base


def test_estimate_rejects_bad_sizes():
    import pcd

    with pytest.raises(pcd.PcdError):
        pcd.estimate_device_bytes(-1, 10, 2)
    with pytest.raises(pcd.PcdError):
        pcd.estimate_device_bytes(10, 10, 2, num_graphs=0)


def test_serve_start_rejects_bad_config():
    import ctypes as C

    import pcd

    h = C.c_void_p()
    for bad in (dict(workers=0), dict(max_batch_graphs=0), dict(hbm_budget_bytes=0), dict(max_wait_ms=-1.0),
                dict(large_graph_edges=1 << 5)):
        kw = dict(device=0, workers=1, max_batch_graphs=8, max_batch_edges=1 << 20, hbm_budget_bytes=1 << 30,
                  max_wait_ms=1.0, use_cuda_graph=0, small_graph_edges=1 << 10, large_graph_edges=1 << 20)
        kw.update(bad)
        cfg = pcd._ServeConfig(**kw)
        assert pcd.LIB.pcd_serve_start(C.byref(cfg), C.byref(h)) == 1
