"""The C++ facade (include/lsdg/lsdg.hpp) compiles against the C-ABI and, driven the way the
reference's tracking and mapping threads would drive it, gives the same pose as the Python binding."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import lsdg
import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_facade_tracks_and_maps(monkeypatch):
    # both sides use the same launch shape (the autotuner could otherwise pick different ones per
    # context, which changes the reduction order and the last bits of the pose)
    monkeypatch.setenv("LSDG_TRACK_SHAPE", "256,8,2")
    p = synth.tracking_pair(21, 320, 240)
    with tempfile.TemporaryDirectory() as d:
        for name, arr in (("key", p.ref_image), ("idepth", p.ref_idepth), ("var", p.ref_idepth_var), ("cur", p.new_image)):
            np.ascontiguousarray(arr, np.float32).tofile(os.path.join(d, name + ".f32"))
        exe = os.path.join(d, "facade_check")
        libdir = os.path.dirname(lsdg.LIB_PATH)
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                               os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-L", libdir, "-llsdg",
                               "-Wl,-rpath," + libdir, "-o", exe])
        out = subprocess.run([exe, d], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.split("\n")
    vals = lines[0].split()
    assert vals[0] == "pose"
    T_cpp = np.array([float(v) for v in vals[1:13]]).reshape(3, 4)
    assert vals[13:15] == ["good", "1"]
    ctx = lsdg.Context()
    kf = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.ref_image).set_depth(p.ref_idepth, p.ref_idepth_var)
    fr = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.new_image)
    T_py, st = lsdg.SE3Tracker(ctx).trackFrame(kf, fr)
    a, t = synth.pose_error(T_cpp, T_py)
    assert a < 1e-7 and t < 1e-7, (a, t)
    assert int(lines[1].split()[1]) > 1000  # depth_valid
