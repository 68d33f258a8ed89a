"""Build recipe for the CPU oracle (test infrastructure only): compiles oracle/*.cpp with g++ twice.

oracle/liblsdo.so, the parity oracle: -O2, -ffp-contract=off so that a*b + c is never fused into an
FMA (the bit-exact CUDA kernels are compiled with -fmad=false for the same reason: the float oracle
and those kernels then round every operation identically), no -ffast-math, the default instruction
set (the same source gives the same results on x86_64 and aarch64 hosts).

oracle/liblsdo_fast.so, the timed CPU baseline: the same sources with -O3, FMA contraction allowed
and code scheduled for the benchmark host's cores (-mtune=neoverse-v2 for the Grace cores of an
aarch64 GB300 host, on the base Armv8-A instruction set with NEON; other hosts keep their default
target).  It stands in for the
upstream CPU path's SSE build flags (CMakeLists.txt:57-59).  Its results differ from the parity
build in the last bits and are only ever checked by tolerance against the FP64 oracle.

The reference's own lsd-slam sources are not present (unvendored fips import, fips.yml:2-4), so
there is no oracle/_ref build of the tracker or the depth filter.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["lsdo_params.cpp", "lsdo_track.cpp", "lsdo_depth.cpp", "lsdo_sim3.cpp", "lsdo_energy.cpp", "lsdo_cloud.cpp", "lsdo_input.cpp"]
LIB = os.path.join(HERE, "liblsdo.so")
FAST_LIB = os.path.join(HERE, "liblsdo_fast.so")

PARITY_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
COMMON = ["-std=c++17", "-fPIC", "-shared", "-pthread", "-Wall", "-Wno-unused-function"]


def fast_flags() -> list:
    flags = ["-O3", "-ffp-contract=fast", "-fno-math-errno", "-funroll-loops"]
    if platform.machine() in ("aarch64", "arm64"):
        # scheduled for the Grace cores, on the base Armv8-A instruction set with NEON: a build for
        # the full neoverse-v2 target (-mcpu) stopped with SIGILL on a GB300 host whose cores do not
        # expose every extension of that target
        flags.append("-mtune=neoverse-v2")
    return flags


def _up_to_date(lib: str, deps) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _build(lib: str, flags: list, force: bool) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "lsdo.h"), os.path.join(HERE, "..", "include", "lsdg.h"), os.path.abspath(__file__)]
    if not force and _up_to_date(lib, deps):
        return lib
    cmd = ["g++"] + COMMON + flags + ["-o", lib + ".tmp"] + srcs
    subprocess.check_call(cmd)
    os.replace(lib + ".tmp", lib)
    return lib


def build(force: bool = False) -> str:
    return _build(LIB, PARITY_FLAGS, force)


_fast_used = None


def build_fast(force: bool = False) -> str:
    global _fast_used
    try:
        _fast_used = fast_flags()
        return _build(FAST_LIB, _fast_used, force)
    except subprocess.CalledProcessError:
        # a compiler that does not know the named core: the same build without the tuning
        _fast_used = [f for f in fast_flags() if not f.startswith("-mtune")]
        return _build(FAST_LIB, _fast_used, True)


def fast_flags_used() -> list:
    """The flags liblsdo_fast.so was built with in this process (after build_fast)."""
    return list(_fast_used if _fast_used is not None else fast_flags())


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_fast(force="--force" in sys.argv))
