"""Pose wire formats (host functions of the library, no GPU): Sophus' 7-float Sim3 layout of
GraphFramePose and the rows of TextOutputIOWrapper's pose file."""
import math

import numpy as np
import pytest

import lsdg
import synth


def p13(R, t, s):
    return np.concatenate([np.asarray(R, np.float64).ravel(), np.asarray(t, np.float64), [s]])


def test_identity_and_known_rotation():
    np.testing.assert_array_equal(lsdg.sim3_to_sophus7(p13(np.eye(3), [0, 0, 0], 1.0)), [0, 0, 0, 1, 0, 0, 0])
    Rz = synth.rodrigues(np.array([0.0, 0.0, math.pi / 2]))
    q = lsdg.sim3_to_sophus7(p13(Rz, [1, 2, 3], 4.0))
    # unit quaternion (0, 0, sin 45, cos 45) scaled by sqrt(4) = 2 (squared norm = scale)
    np.testing.assert_allclose(q, [0, 0, 2 * math.sin(math.pi / 4), 2 * math.cos(math.pi / 4), 1, 2, 3], atol=1e-6)


@pytest.mark.parametrize("seed", range(6))
def test_round_trip(seed):
    rng = np.random.default_rng(seed)
    axis = rng.normal(size=3)
    angle = rng.uniform(0, math.pi) if seed % 2 else rng.uniform(2.5, math.pi)  # includes near-pi
    R = synth.rodrigues(axis / np.linalg.norm(axis) * angle)
    s = float(rng.uniform(0.2, 5.0))
    t = rng.normal(size=3)
    q = lsdg.sim3_to_sophus7(p13(R, t, s))
    assert q[3] >= 0
    assert float(np.dot(q[:4].astype(np.float64), q[:4])) == pytest.approx(s, rel=1e-6)
    back = lsdg.sophus7_to_sim3(q)
    np.testing.assert_allclose(back[:9], R.ravel(), atol=2e-6)
    np.testing.assert_allclose(back[9:12], t.astype(np.float32), rtol=0, atol=0)
    assert back[12] == pytest.approx(s, rel=1e-6)


def test_pose_row_like_an_ostream():
    c = p13(np.eye(3), [1.5, -2.0, 0.125], 1.0)
    t = p13(np.eye(3), [0.0, 1e-7, 123456789.0], 1.0)
    assert lsdg.format_pose_row(7, c, t) == "7,1.5,-2,0.125,0,1e-07,1.23457e+08\n"


def test_graph_frame_pose_layout():
    import ctypes as C

    class GraphFramePose(C.Structure):
        _fields_ = [("id", C.c_int32), ("cam_to_world", C.c_float * 7)]
    assert C.sizeof(GraphFramePose) == 32
