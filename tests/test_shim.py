"""The shim that replaces the reference's GPU host API
(src/framework-cuda.cuh:14-23) with libpcd compiles and links against the
reference's own Graph (graph.hpp, graph.o built from the reference sources)
and against the stand-in Graph used where those sources are absent.  Its run
on the device is tests/test_gpu_shim.py."""
import os

import pytest


def test_shim_builds_against_the_reference_graph(tmp_path):
    import shim_build

    src, _ = shim_build.reference_src()
    if src is None:
        pytest.skip("reference sources or oracle/_ref not present")
    inc = shim_build.build(os.path.join(tmp_path, "shim_ref"), use_reference=True)
    assert inc == src


def test_shim_builds_against_the_stand_in_graph(tmp_path):
    import shim_build

    shim_build.build(os.path.join(tmp_path, "shim_stand_in"), use_reference=False)
