"""CPU: the C-ABI library builds, loads, and exports every entry point that
include/pcd.h declares; host-side logic (seed stream, initial partitions)
matches libc and the oracle; calls fail with status codes, not crashes."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT, golden_graph


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "pcd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pcd_[a-z_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    import build

    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_and_no_gpu_init():
    import pcd

    for s in range(8):
        assert pcd.LIB.pcd_status_string(s)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        try:
            pcd.Context(0)
        except pcd.PcdError as e:
            assert e.status in (2, 3)  # a CUDA error code, not a crash
        else:  # pragma: no cover
            raise AssertionError("pcd_init succeeded without a device")


def test_host_seed_stream_matches_libc():
    import pcd

    libc = ctypes.CDLL("libc.so.6")
    libc.rand.restype = ctypes.c_int
    libc.srand(1)
    want = [libc.rand() for _ in range(4000)]
    r = pcd.GlibcRand()
    assert [r() for _ in range(4000)] == want
    r2 = pcd.GlibcRand()
    r2.skip(1234)
    libc.srand(1)
    for _ in range(1234):
        libc.rand()
    assert r2() == libc.rand()


def test_host_initial_partitions_match_oracle(port):
    import pcd

    for name in ("rmat12", "pl20k"):
        g = golden_graph(name)
        port.load(g.indices, g.adj)
        port.srand(1)
        want = port.singleton()

        class Fake:  # a graph handle is only needed for n on this path
            n = g.n

            class ctx:
                @staticmethod
                def _check(st):
                    assert st == 0

        got = pcd.create_singleton_partition(Fake, pcd.GlibcRand())
        assert np.array_equal(got, want)
        tri, _, _ = port.count_triangles()
        lab = np.zeros(g.n, np.int32)
        st = pcd.LIB.pcd_clustering_partition(g.n, pcd._ptr(g.indices), pcd._ptr(g.adj), pcd._ptr(tri), pcd._ptr(lab))
        assert st == 0
        assert np.array_equal(lab, port.clustering())


def declared_arity():
    """Parameter count of every function declared in include/pcd.h."""
    text = open(os.path.join(ROOT, "include", "pcd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(pcd_[a-z_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_python_bindings_match_the_header():
    """Every function pcd.py binds takes as many arguments as the header
    declares (a wrong count would pass garbage through ctypes)."""
    import pcd

    arity = declared_arity()
    bound = [n for n in dir(pcd.LIB) if n.startswith("pcd_")]
    assert len(bound) >= 20
    for name in bound:
        f = getattr(pcd.LIB, name)
        if f.argtypes is None:
            continue
        assert name in arity, f"{name} is bound but not declared"
        assert len(f.argtypes) == arity[name], (name, len(f.argtypes), arity[name])
