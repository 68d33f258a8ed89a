"""Build recipe for oracle/_ref (test infrastructure only): the reference's own point-cloud loop,
Keyframe::computeVbo (lib/Pangolin_IOWrapper/Keyframe.h:66-143), compiled from its source as a CPU
checker of the cloud kernel and of the cloud oracle.

Keyframe.h is a header of the OpenGL viewer: it includes GLEW and Sophus (both absent) and ends
computeVbo with a GL buffer upload.  The recipe therefore compiles no GL at all: it reads the header
where it lies, takes from it, unchanged, the declaration of InputPointDense (:16-21), the
declaration of Keyframe::MyVertex (:50-54) and the body of computeVbo from its vertex buffer
allocation (:75) up to the first GL call after the loop (:145), and wraps that text in a harness
whose members carry the names the body uses (width, height, fx, fy, cx, cy, pointData, points, and
camToWorld with a scale() accessor for the float scale of the keyframe's Sim3).  The harness and
the compiled library are written to oracle/_ref/ only (git-ignored).  The flags are the
reference's release flags without its x86 ISA switches (CMakeLists.txt:57-63: -std=c++11 -O3;
ISO C++ mode, so no FMA contraction, which -ffp-contract=off states explicitly).

The generated source travels with the repository copy; where the reference tree is absent but the
generated source is present, the library is compiled from it.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
KEYFRAME_H = "/root/reference/lib/Pangolin_IOWrapper/Keyframe.h"
SRC = os.path.join(OUT, "computevbo_ref.cpp")
LIB = os.path.join(OUT, "libcomputevbo_ref.so")
FLAGS = ["-std=c++11", "-O3", "-DNDEBUG", "-ffp-contract=off", "-fPIC", "-shared"]


def _block(lines, start_pat, what):
    """Lines of the first brace block whose opening line matches start_pat, through its '};'."""
    for i, ln in enumerate(lines):
        if re.search(start_pat, ln):
            for j in range(i, len(lines)):
                if lines[j].strip() == "};":
                    return lines[i:j + 1]
    raise RuntimeError(f"{what} not found in Keyframe.h")


def extract(text: str) -> dict:
    lines = text.splitlines()
    point = _block(lines, r"^struct InputPointDense\b", "InputPointDense")
    vertex = _block(lines, r"^\s*struct MyVertex\b", "Keyframe::MyVertex")
    fn = next(i for i, ln in enumerate(lines) if re.search(r"void computeVbo\(\)", ln))
    begin = next(i for i in range(fn, len(lines)) if "new MyVertex" in lines[i])
    end = next(i for i in range(begin, len(lines)) if re.search(r"\bgl[A-Z]\w*\s*\(", lines[i]))
    body = lines[begin:end]
    joined = "\n".join(body)
    if re.search(r"\bgl[A-Z]\w*|\bGL_", joined) or "for(int y" not in joined.replace(" (", "("):
        raise RuntimeError("unexpected computeVbo body in Keyframe.h")
    return {"point": point, "vertex": vertex, "body": body}


HARNESS = """// Generated by oracle/ref_build.py from the reference's Keyframe.h (not committed): the
// declarations of InputPointDense and Keyframe::MyVertex and computeVbo's filter and
// back-projection loop, unchanged, inside a harness without OpenGL.
#include <cassert>
#include <cstdlib>
#include <cstring>

{point}

namespace refvbo {{
struct Sim3Scale {{
  float s;
  float scale() const {{ return s; }}
}};

struct Harness {{
{vertex}
  Sim3Scale camToWorld;
  float fx, fy, cx, cy;
  int height, width;
  unsigned char* pointData;
  int points;

  MyVertex* loop() {{
{body}
    return tmpBuffer;
  }}
}};
}}  // namespace refvbo

extern "C" int ref_compute_vbo(int w, int h, float fx, float fy, float cx, float cy, float scale,
                               const void* points, void* out) {{
  refvbo::Harness k;
  k.width = w;
  k.height = h;
  k.fx = fx;
  k.fy = fy;
  k.cx = cx;
  k.cy = cy;
  k.camToWorld.s = scale;
  k.pointData = (unsigned char*)points;
  k.points = 0;
  refvbo::Harness::MyVertex* v = k.loop();
  std::memcpy(out, v, sizeof(*v) * (size_t)k.points);
  delete[] v;
  return k.points;
}}

extern "C" int ref_sizes(int* point_dense, int* vertex) {{
  *point_dense = (int)sizeof(InputPointDense);
  *vertex = (int)sizeof(refvbo::Harness::MyVertex);
  return 0;
}}
"""


def generate(keyframe_h: str = KEYFRAME_H) -> str:
    with open(keyframe_h) as f:
        parts = extract(f.read())
    src = HARNESS.format(point="\n".join(parts["point"]), vertex="\n".join(parts["vertex"]),
                         body="\n".join(parts["body"]))
    os.makedirs(OUT, exist_ok=True)
    with open(SRC + ".tmp", "w") as f:
        f.write(src)
    os.replace(SRC + ".tmp", SRC)
    return SRC


def build(force: bool = False):
    """Path of oracle/_ref/libcomputevbo_ref.so, or None when neither the reference tree nor a
    generated source is present."""
    if os.path.exists(KEYFRAME_H):
        if force or not os.path.exists(SRC) or os.path.getmtime(SRC) < max(
                os.path.getmtime(KEYFRAME_H), os.path.getmtime(os.path.abspath(__file__))):
            generate()
    elif not os.path.exists(SRC):
        return None
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["g++"] + FLAGS + ["-o", LIB + ".tmp", SRC])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
