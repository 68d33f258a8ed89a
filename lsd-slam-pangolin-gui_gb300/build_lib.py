"""Build recipe of the product library liblsdg.so (CUDA sm_103a + C-ABI), in-tree.

Each csrc/*.cu is compiled by nvcc in parallel (one -gencode, compute_103a -> sm_103a) and linked
into lsd-slam-pangolin-gui_gb300/liblsdg.so.  Kernels are built with -fmad=false (every float
operation rounds on its own, exactly like the CPU oracle built with -ffp-contract=off, which is what
makes pyramids, points and depth-filter decisions bit-identical to it), except the tracker, which
is built with FMA contraction (see FMAD).  The rebuild is triggered by source or header changes and
by a change of this file.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblsdg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE]
# (host code too is built without FMA contraction: the per-reference geometry the depth filter
# derives from a pose in double must round to the same floats as the CPU oracle's on any host)
# Translation units whose float results must be bit-identical to the CPU oracle are built without
# FMA contraction; the tracker (parity by tolerance, throughput-critical) is built with it.
FMAD = {"track.cu": "-fmad=true"}


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, "lsdg.h")]


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + headers() + [os.path.abspath(__file__)]
    if os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in deps):
        return obj
    fmad = FMAD.get(os.path.basename(src), "-fmad=false")
    cmd = [NVCC] + GENCODE + FLAGS + [fmad] + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + GENCODE + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
