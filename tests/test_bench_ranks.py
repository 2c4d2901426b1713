"""CPU: bench.py's host-side rules -- the multi-rank path with the gloo
backend (world size 2), the reference schedule's seeds and the per-class
algorithmic bytes.

The sweep has no exchange step, so ranks run independent replicas; what the
ranks share is the timing rule (the job's time is the slowest rank's) and
one printed line.  Both are exercised here without a GPU: the max-over-ranks
helper in two gloo processes, and the reference arm under torchrun, where
rank 0 alone runs and prints and rank 1 exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(dist, 1.0 + 2.0 * rank, "cpu")
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write(repr(got))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(None, 2.5, "cpu") == 2.5
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    assert [float((tmp_path / f"r{r}").read_text()) for r in (0, 1)] == [3.0, 3.0]


def test_reference_arm_two_ranks_prints_one_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "12", "--steps", "1", "--warmup", "0",
           "--sweeps", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")


def test_schedule_seeds_are_the_reference_drivers():
    """The bench replays the reference schedule's sweeps: the seed of sweep i
    is the (n + i + 1)-th value of glibc rand() after srand(1) (the singleton
    partition draws n first, src/framework.cpp:14-24; each refinement draws
    one, src/refinement.cpp:123-124)."""
    import ctypes

    sys.path.insert(0, ROOT)
    import bench

    import numpy as np

    libc = ctypes.CDLL("libc.so.6")
    libc.rand.restype = ctypes.c_int
    for n in (0, 1, 1000, 123457):
        libc.srand(ctypes.c_uint(1))
        for _ in range(n):
            libc.rand()
        ind = np.zeros(n + 1, np.int32)  # n isolated vertices: only n matters
        assert bench.schedule_seeds(ind, np.zeros(0, np.int32), 5) == [libc.rand() for _ in range(5)]


def test_reference_arm_helpers_map_no_product_library():
    """The reference arm draws its seeds and runs its sweeps through the
    oracle only: libpcd.so is never mapped into that process."""
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r); import bench, graphs; "
        "g = graphs.convert_edges(graphs.rmat(10, 8, 0.57, 0.19, 0.19, seed=2)); "
        "s = bench.schedule_seeds(g.indices, g.adj, 2); "
        "bench.cpu_sweeps(g.indices, g.adj, s, 2, 2, 10.0); "
        "maps = open('/proc/self/maps').read(); "
        "print('libpcd.so' in maps, 'libpcd_oracle.so' in maps)" % ROOT)
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "par-cd_gb300"),
                                                       os.path.join(ROOT, "oracle")]))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.split() == ["False", "True"], r.stdout


def test_bins_bytes_sum_to_the_sweep_formula():
    """Per-class algorithmic bytes (8 per endpoint + 12 per vertex) add up to
    the sweep's 16m + 12n (+4 for the last row offset, counted once)."""
    import numpy as np

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "par-cd_gb300"))
    import bench
    import graphs

    g = graphs.convert_edges(graphs.rmat(12, 16, 0.57, 0.19, 0.19, seed=2))
    bb = bench.bins_bytes(g.indices)
    assert sum(bb.values()) + 4 == 16 * g.m + 12 * g.n + 4
    assert set(bb) == {"sweep.g4", "sweep.g8", "sweep.g16", "sweep.g32", "sweep.warp", "sweep.block",
                       "sweep.block_l", "sweep.hub"}
