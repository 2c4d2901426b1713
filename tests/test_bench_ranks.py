"""CPU: the multi-rank path of bench.py with the gloo backend (world size 2).

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
