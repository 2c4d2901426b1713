"""Builds tests/shim/framework_cuda_pcd.cpp (the reference's GPU host API
over libpcd, with a small schedule driver): against the reference's own
graph.hpp and graph.o where the reference sources and the oracle/_ref build
are present, else against the stand-in Graph of tests/shim/graph_stand_in."""
import os
import subprocess

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SHIM = os.path.join(ROOT, "tests", "shim", "framework_cuda_pcd.cpp")
PKG = os.path.join(ROOT, "par-cd_gb300")


def reference_src():
    src = os.environ.get("PCD_REFERENCE_SRC", "/root/reference/src")
    obj = os.path.join(ROOT, "oracle", "_ref", "strict", "graph.o")
    if os.path.isfile(os.path.join(src, "graph.hpp")) and os.path.isfile(obj):
        return src, obj
    return None, None


def build(out, use_reference=None):
    """Compiles and links the shim driver to `out`; returns the Graph header
    directory used."""
    src, obj = reference_src()
    if use_reference is None:
        use_reference = src is not None
    inc = src if use_reference else os.path.join(ROOT, "tests", "shim", "graph_stand_in")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", inc, "-I", os.path.join(ROOT, "include"), SHIM]
    if use_reference:
        cmd += [obj, "-fopenmp"]
    cmd += ["-L", PKG, "-lpcd", f"-Wl,-rpath,{PKG}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shim build failed:\n{' '.join(cmd)}\n{r.stderr}")
    return inc
