"""In-tree build of libolgpu.so (sm_103a) and of the Olliptic.x drop-in CLI.

The CUDA translation unit and the host geometry are compiled in parallel and
linked by nvcc.  Host code is built with -ffp-contract=off: the hierarchy's
coordinates must round exactly like the reference's so that the same coarse
and fine points coincide on x86-64 and on aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(BUILD, "libolgpu.so")
CLI = os.path.join(BUILD, "Olliptic_gpu.x")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")

CU_SOURCES = ["olgpu.cu"]
CPP_SOURCES = ["grid.cpp", "server.cpp"]
HEADERS = ["device.cuh", "kernels.cuh", "coarse_cluster.cuh", "mixed.cuh", "smooth_cluster.cuh", "grid.h", "../../include/olgpu.h"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libolgpu.so (and the CLI) if any source changed; return the .so path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES + HEADERS]
    cli_src = os.path.join(CSRC, "olliptic_cli.cpp")
    if not force and not _stale(LIB, srcs) and (not os.path.exists(cli_src) or not _stale(CLI, [cli_src, LIB])):
        return LIB
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        jobs.append([NVCC, "-O3", "-std=c++17", "-c", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     *ARCH, "-lineinfo", "-I", INCLUDE, os.path.join(CSRC, s), "-o", o])
    for s in CPP_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-I", INCLUDE, "-c",
                     os.path.join(CSRC, s), "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    _run([NVCC, "-shared", *ARCH, *objs, "-o", LIB, "-lcudart", "-lpthread"])
    if os.path.exists(cli_src):
        _run([CXX, "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, cli_src, "-o", CLI,
              "-L", BUILD, "-lolgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
