"""The drop-in driver (par-cd_gb300/main-cuda): the reference CPU driver's
command line and output, with every phase on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_graph

MAIN = os.path.join(ROOT, "par-cd_gb300", "main-cuda")


def _built():
    import build

    build.build()
    return MAIN


def test_main_cuda_rejects_bad_flags():
    exe = _built()
    for argv in ([], ["g.bin", "-m", "nope"], ["g.bin", "-f", "0"], ["g.bin", "-r", "0"], ["g.bin", "-t", "2"]):
        r = subprocess.run([exe] + argv, capture_output=True, text=True)
        assert r.returncode == 255, argv


def test_main_cuda_rejects_missing_or_corrupt_file(tmp_path):
    exe = _built()
    r = subprocess.run([exe, str(tmp_path / "missing.bin")], capture_output=True, text=True)
    assert r.returncode == 255 and "failed to open" in r.stderr
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"PCD\x05\x00\x00\x00")
    r = subprocess.run([exe, str(bad)], capture_output=True, text=True)
    assert r.returncode == 255


@pytest.mark.gpu
@pytest.mark.parametrize("args,metric,strategy,rounds,n_iter,initial", [
    (["-m", "mod", "-s", "2", "-n", "12", "-f", "1.0"], "mod", 2, 1, 12, 0),
    (["-m", "cpm-0.01", "-s", "0", "-n", "6", "-f", "0.5"], "cpm-0.01", 0, 1, 6, 0),
    (["-m", "wcc", "-s", "2", "-n", "4", "-i", "1", "-f", "1.0", "-r", "2"], "wcc", 2, 2, 4, 1),
])
def test_main_cuda_matches_oracle(tmp_path, port, args, metric, strategy, rounds, n_iter, initial):
    import graphs
    import oracle

    exe = _built()
    g = golden_graph("sbm10k") if metric != "wcc" else golden_graph("pl20k")
    path = tmp_path / "g.bin"
    graphs.write_pcd(str(path), g)
    r = subprocess.run([exe, str(path)] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 1, r.stderr[-2000:]  # the reference driver exits with 1
    frac = float(args[args.index("-f") + 1])
    final, score, sweeps = oracle.run_schedule(port, g.indices, g.adj, metric, strategy, frac, rounds, n_iter, 0.0,
                                               initial)
    dump = np.array([list(map(int, ln.split())) for ln in r.stderr.strip().splitlines()], dtype=np.int64)
    assert np.array_equal(dump[:, 0], g.map)
    assert np.array_equal(dump[:, 1], final)
    assert f"iteration {n_iter + 1}:" in r.stdout
    assert f"num. communities: {int(final.max()) + 1}" in r.stdout


def test_convert_cuda_rejects_bad_input(tmp_path):
    import build

    build.build()
    exe = os.path.join(ROOT, "par-cd_gb300", "convert-cuda")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 255
    bad = tmp_path / "bad.txt"
    bad.write_text("1 2\n3 x\n")
    r = subprocess.run([exe, str(bad), str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 255 and "line 2 is corrupt" in r.stderr
    r = subprocess.run([exe, str(tmp_path / "missing.txt"), str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 255
