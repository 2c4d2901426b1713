"""The allocation-free relabelling entry point, through the C ABI.

pcd_compress_labels_noalloc is for callers that cannot allocate device
memory at the point where they relabel (for example code running inside
another framework's memory arena, or a serving loop that must not hit
cudaMalloc's device synchronisation).  It keeps its scratch in a fixed
device array instead.  This file checks it against pcd_compress (the entry
point that allocates when a graph is loaded) on two calls in a row, so that
the second call sees the array exactly as the first call left it.  It is
collected last, and it needs nothing from the other test files.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, os.path.join(ROOT, "par-cd_gb300"))

pytestmark = pytest.mark.gpu


def _reference_compress(pcd, ctx, labels):
    """Relabel through the allocating path: a graph of n isolated vertices."""
    n = labels.shape[0]
    g = pcd.Graph.from_csr(ctx, np.zeros(n + 1, np.int32), np.zeros(0, np.int32))
    g.labels = labels
    k = g.compress()
    out = g.labels
    g.free()
    return out, k


def test_noalloc_matches_allocating_compress_twice_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pcd

    lib = pcd.LIB
    lib.pcd_compress_labels_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.pcd_compress_labels_noalloc.restype = C.c_int32
    maxn = 1 << 20
    torch.cuda.set_device(0)
    ctx = pcd.Context(0)
    rng = np.random.default_rng(123)
    stream = torch.cuda.current_stream()
    cases = [
        (300_000, 5_000, 0.05),   # many labels shared, some NEW_LABEL
        (maxn, 900_000, 0.2),     # the maximum size, sparse reuse
    ]
    for n, span, p_new in cases:
        lab = rng.integers(0, span, size=n).astype(np.int32)
        lab[rng.random(n) < p_new] = -1
        d_in = torch.from_numpy(lab).cuda()
        d_out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
        st = lib.pcd_compress_labels_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), d_k.data_ptr(),
                                             C.c_void_p(stream.cuda_stream))
        assert st == 0
        torch.cuda.synchronize()
        want, k = _reference_compress(pcd, ctx, lab)
        assert int(d_k.item()) == k
        assert np.array_equal(d_out.cpu().numpy(), want)
    # labels outside [-1, n) take a fresh id each, like NEW_LABEL (-1)
    n = 50_000
    lab = rng.integers(0, 2_000, size=n).astype(np.int32)
    odd = rng.random(n)
    lab[odd < 0.03] = n + rng.integers(0, 1000, size=int((odd < 0.03).sum())).astype(np.int32)
    lab[(odd >= 0.03) & (odd < 0.06)] = -2 - rng.integers(0, 1000, size=int(((odd >= 0.03) & (odd < 0.06)).sum()))
    lab[(odd >= 0.06) & (odd < 0.08)] = -1
    lab[:3] = [n, -5, 2**31 - 1]
    d_in = torch.from_numpy(lab).cuda()
    d_out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.pcd_compress_labels_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), d_k.data_ptr(),
                                           C.c_void_p(stream.cuda_stream)) == 0
    torch.cuda.synchronize()
    as_new = np.where((lab < -1) | (lab >= n), -1, lab).astype(np.int32)
    want, k = _reference_compress(pcd, ctx, as_new)
    assert int(d_k.item()) == k
    assert np.array_equal(d_out.cpu().numpy(), want)
    # n == 0: no labels, a count of 0 written on the stream
    d_k.fill_(-3)
    assert lib.pcd_compress_labels_noalloc(None, 0, None, d_k.data_ptr(), C.c_void_p(stream.cuda_stream)) == 0
    torch.cuda.synchronize()
    assert int(d_k.item()) == 0
    # sizes beyond the fixed array are refused without touching the outputs
    big = torch.zeros(maxn + 1, dtype=torch.int32, device="cuda")
    out = torch.zeros(maxn + 1, dtype=torch.int32, device="cuda")
    kk = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.pcd_compress_labels_noalloc(big.data_ptr(), maxn + 1, out.data_ptr(), kk.data_ptr(), None) == 1
    ctx.close()
