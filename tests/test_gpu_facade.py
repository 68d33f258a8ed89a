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
    sp = synth.sim3_pair(22, 320, 240)
    with tempfile.TemporaryDirectory() as d:
        for name, arr in (("key", p.ref_image), ("idepth", p.ref_idepth), ("var", p.ref_idepth_var), ("cur", p.new_image),
                          ("s_key", sp.ref_image), ("s_kid", sp.ref_idepth), ("s_kvar", sp.ref_idepth_var),
                          ("s_new", sp.new_image), ("s_nid", sp.new_idepth), ("s_nvar", sp.new_idepth_var)):
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
    # energy: the same kernels on the same inputs -> the same numbers
    ev = lines[2].split()
    assert ev[0] == "energy"
    en = lsdg.PhotometricEnergy(ctx, kf, 0)
    E = en.forward(fr, synth.pose_inv(T_cpp))
    gxi, grho = en.backward(1.0)
    en.close()
    assert float(ev[1]) == pytest.approx(E, rel=1e-12)
    np.testing.assert_allclose([float(v) for v in ev[2:8]], gxi, rtol=1e-12)
    assert int(ev[9]) == len(grho) and int(ev[11]) == int(np.count_nonzero(grho))
    # Sim3 tracking through the facade vs the Python binding
    sv = lines[3].split()
    assert sv[0] == "sim3" and sv[14:16] == ["good", "1"]
    ki = lsdg.Frame(ctx, sp.w, sp.h, sp.intr).upload(sp.ref_image).set_depth(sp.ref_idepth, sp.ref_idepth_var)
    kj = lsdg.Frame(ctx, sp.w, sp.h, sp.intr).upload(sp.new_image).set_depth(sp.new_idepth, sp.new_idepth_var)
    (Ts, ss), _ = lsdg.Sim3Tracker(ctx).trackFrameSim3(ki, kj)
    got = np.array([float(v) for v in sv[1:14]])
    np.testing.assert_allclose(got[:12], np.concatenate([Ts[:, :3].ravel(), Ts[:, 3]]), rtol=0, atol=1e-7)
    assert got[12] == pytest.approx(ss, abs=1e-7)
