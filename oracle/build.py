"""Build recipe for the CPU oracle (test infrastructure only): compiles oracle/*.cpp into
oracle/liblsdo.so with g++.

Flags: -O2 for speed, -ffp-contract=off so that a*b + c is never fused into an FMA (the CUDA
kernels are compiled with -fmad=false for the same reason: the float oracle and the kernels then
round every operation identically), no -ffast-math, no -march=native (the same source builds on
x86_64 and aarch64 hosts).  The reference's own lsd-slam sources are not present (unvendored fips
import, fips.yml:2-4), so there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["lsdo_params.cpp", "lsdo_track.cpp", "lsdo_depth.cpp", "lsdo_sim3.cpp", "lsdo_energy.cpp", "lsdo_cloud.cpp", "lsdo_input.cpp"]
LIB = os.path.join(HERE, "liblsdo.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "lsdo.h"), os.path.join(HERE, "..", "include", "lsdg.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"] + srcs
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
