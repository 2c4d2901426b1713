"""Build recipe for libpcd.so (in-tree, sm_103a only).

Every translation unit is compiled in parallel with nvcc for
`-gencode arch=compute_103a,code=sm_103a` and linked into
par-cd_gb300/libpcd.so; the drop-in driver par-cd_gb300/main-cuda links it.  `-fmad=false` keeps FP64 products and sums from
being contracted into FMAs, so device gains are the IEEE results of the
reference's own operation sequence.

    python par-cd_gb300/build.py [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpcd.so")
MAIN = os.path.join(HERE, "main-cuda")
CONVERT = os.path.join(HERE, "convert-cuda")
SOURCES = ["api.cu", "partition.cu", "propagate.cu", "merge.cu", "triangles.cu", "batch.cu", "noalloc.cu", "convert.cu", "components.cu", "initial.cu", "nmi.cu", "hostside.cpp", "serve.cpp"]
HEADERS = ["pcd_device.cuh", "pcd_scan.cuh", "pcd_internal.h", "pcd_types.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-O2",
                   "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")] + list(extra)


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "pcd.h")]
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        if force or _stale(o, [s] + hdrs + [__file__]):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        if s.endswith(".cpp"):
            cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
            cmd = ["g++", "-c", s, "-o", o, "-O2", "-fPIC", "-std=c++17", "-pthread", "-ffp-contract=off",
                   "-fno-fast-math", "-I", os.path.join(HERE, "..", "include"), "-I", cuda_inc, "-I", CSRC]
        else:
            cmd = [nvcc(), "-c", s, "-o", o] + flags(extra)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stderr}")
        return r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for msg in ex.map(compile_one, jobs):
                if verbose and msg:
                    print(msg)
    objs = [os.path.join(BUILD, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC,-pthread", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    for exe, src in ((MAIN, "main_cuda.cpp"), (CONVERT, "convert_cuda.cpp")):
        src = os.path.join(CSRC, src)
        if force or _stale(exe, [src, LIB]):
            cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"), "-o", exe, src, "-L",
                   HERE, "-lpcd", "-Wl,-rpath,$ORIGIN"]
            if verbose:
                print(" ".join(cmd), flush=True)
            subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
