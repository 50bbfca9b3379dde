"""Build libbfgpu.so in-tree for sm_103a (nvcc + g++, no cmake).

Usage: ``python butterflyfactorizations.jl_gb300/build_ext.py [--force]``.
Objects go to ``butterflyfactorizations.jl_gb300/build/``, the library to
``butterflyfactorizations.jl_gb300/bfgpu/libbfgpu.so``.  Translation units are
compiled in parallel and skipped when newer than their sources and headers.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "bfgpu", "libbfgpu.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(INCLUDE, "bfgpu.h"))
    return srcs, hdrs


def _cmd(src: str, obj: str):
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        return [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                "-Xptxas", "-warn-spills", "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", obj]
    # -ffp-contract=off: no fused multiply-adds in host code, so the FP64 tests of the
    # tree traversal round the same on x86-64, aarch64 and in the device version
    return ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-fvisibility=hidden",
            "-Wall",
            "-Wno-unused-function", "-I", INCLUDE, "-I", CSRC, "-I",
            os.path.join(CUDA, "include"), "-fopenmp", "-c", path, "-o", obj]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs, hdrs = _sources()
    hdr_time = max(os.path.getmtime(h) for h in hdrs)
    jobs = []
    objs = []
    for s in srcs:
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or \
                os.path.getmtime(obj) < max(os.path.getmtime(os.path.join(CSRC, s)), hdr_time):
            jobs.append((s, obj))

    def run(job):
        s, obj = job
        cmd = _cmd(s, obj)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for s, r in ex.map(run, jobs):
                if r.returncode != 0:
                    raise RuntimeError(f"compiling {s} failed:\n{r.stdout}\n{r.stderr}")
                if verbose and (r.stderr.strip()):
                    print(r.stderr, flush=True)
    if force or jobs or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs,
               "-Xcompiler", "-fopenmp", "-lgomp", "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
