"""Builds the CUDA library (libkcna.so) in-tree for sm_103a with nvcc.

Each .cu translation unit is compiled in parallel, then linked into
fastkcna_gb300/libkcna.so.  Object files go to fastkcna_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkcna.so")
SOURCES = ["kcna_api.cu", "kcna_knn.cu", "kcna_nnd.cu", "kcna_join_tc.cu", "kcna_p2k_tc.cu", "kcna_prune_tc.cu", "kcna_prune_fp8.cu", "kcna_graph.cu", "kcna_noalloc.cu",
           "kcna_tc.cu", "kcna_seed.cu", "kcna_cagra.cu",
           "kcna_pool_search.cu", "kcna_io.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "kcna.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if _stale(obj, src) or ptxas_v:
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append((src, obj, [nvcc(), *flags(extra), "-c", src, "-o", obj]))

    def run(job):
        src, obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src, r in ex.map(run, jobs):
            if verbose or ptxas_v or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}")
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libkcna.so failed")
    build_host(verbose)
    return LIB


HOST = os.path.join(HERE, "host")
FACADE = os.path.join(HERE, "libkgraph_gb300.so")
BIN = os.path.join(HERE, "bin")
TOOLS = {"fastnsg": 1, "fasttaumng": 2, "fastalphapg": 3, "fasthnsw": 4, "fastnsw": 5}


def build_host(verbose: bool = False) -> None:
    """The C++ kgraph::KGraph facade (libkgraph_gb300.so), the five command
    lines (bin/fast*, linked against libkcna.so) and the fvecs converter
    (bin/fvec2lshkit, host code only)."""
    cxx = os.environ.get("CXX", "g++")
    inc = ["-I", os.path.join(ROOT, "include")]
    common = [cxx, "-O2", "-std=c++17", "-Wall", "-Wno-unused-result", *inc]
    facade_src = os.path.join(HOST, "kgraph_facade.cpp")
    cli_src = os.path.join(HOST, "fastkcna_cli.cpp")
    headers = [os.path.join(ROOT, "include", h) for h in ("kcna.h", "kgraph_gb300.h", "kgraph_gb300_data.h")]

    def stale(out, srcs):
        return not os.path.exists(out) or any(os.path.getmtime(x) > os.path.getmtime(out) for x in srcs)

    if stale(FACADE, [facade_src, LIB, *headers]):
        cmd = common + ["-fPIC", "-shared", facade_src, "-o", FACADE, "-L", HERE, "-lkcna",
                        "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("g++ failed on kgraph_facade.cpp")
    os.makedirs(BIN, exist_ok=True)
    jobs = []
    conv_src = os.path.join(HOST, "fvec2lshkit.cpp")
    conv = os.path.join(BIN, "fvec2lshkit")
    if stale(conv, [conv_src]):
        jobs.append(("fvec2lshkit", common + [conv_src, "-o", conv]))
    for tool, k in TOOLS.items():
        out = os.path.join(BIN, tool)
        if stale(out, [cli_src, FACADE, *headers]):
            jobs.append((tool, common + [f"-DKCNA_CLI={k}", cli_src, "-o", out, "-L", HERE, "-lkgraph_gb300",
                                         "-lkcna", "-Wl,-rpath,$ORIGIN/.."]))
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for tool, r in ex.map(lambda j: (j[0], subprocess.run(j[1], capture_output=True, text=True)), jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"g++ failed on {tool}")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_v="--ptxas" in sys.argv))
