"""CPU tests of the input step: the calibration reader (library, host only), the undistortion
oracle against an independent numpy restatement of the model, and known answers (pinhole identity,
pure radial displacement on the axes)."""
import os
import tempfile

import numpy as np
import pytest

import lsdg
import lsdg_types as T
import lsdo

XML = """<?xml version="1.0" encoding="UTF-8"?>
<calibration>
  <projection>frame</projection>
  <width>640</width>
  <height>480</height>
  <f>512.25</f>
  <cx>-6.5</cx>
  <cy>4.25</cy>
  <b2>-1.5</b2>
  <k1>-0.12</k1>
  <k2>0.29</k2>
  <p1>0.0004</p1>
  <p2>0.0018</p2>
</calibration>
"""


def calib_frame():
    c = T.Calibration()
    c.model, c.width, c.height = T.CALIB_FRAME, 640, 480
    c.f, c.cx, c.cy, c.b2 = 512.25, -6.5, 4.25, -1.5
    c.k1, c.k2, c.p1, c.p2 = -0.12, 0.29, 0.0004, 0.0018
    return c


def default_K(c):
    f32 = np.float32
    return T.Intrinsics(f32(c.f), f32(c.f), f32(0.5 * c.width + c.cx - 0.5), f32(0.5 * c.height + c.cy - 0.5))


def numpy_map(c, w, h, K):
    x = (np.arange(w, dtype=np.float64)[None, :] - np.float64(K.cx)) / np.float64(K.fx)
    y = (np.arange(h, dtype=np.float64)[:, None] - np.float64(K.cy)) / np.float64(K.fy)
    x, y = np.broadcast_arrays(x, y)
    r2 = x * x + y * y
    rad = 1.0 + r2 * (c.k1 + r2 * (c.k2 + r2 * (c.k3 + r2 * c.k4)))
    xd = x * rad + (c.p1 * (r2 + 2.0 * x * x) + 2.0 * c.p2 * x * y)
    yd = y * rad + (c.p2 * (r2 + 2.0 * y * y) + 2.0 * c.p1 * x * y)
    u = ((0.5 * c.width + c.cx) + xd * c.f) + (xd * c.b1 + yd * c.b2)
    v = (0.5 * c.height + c.cy) + yd * c.f
    return np.stack([(u - 0.5).astype(np.float32), (v - 0.5).astype(np.float32)], -1)


def test_calibration_xml_reader():
    with tempfile.NamedTemporaryFile("w", suffix=".xml", delete=False) as f:
        f.write(XML)
        path = f.name
    try:
        c = lsdg.calibration_load_xml(path)
    finally:
        os.unlink(path)
    assert c.model == T.CALIB_FRAME and (c.width, c.height) == (640, 480)
    assert (c.f, c.cx, c.cy, c.b1, c.b2) == (512.25, -6.5, 4.25, 0.0, -1.5)
    assert (c.k1, c.k2, c.k3, c.k4, c.p1, c.p2) == (-0.12, 0.29, 0.0, 0.0, 0.0004, 0.0018)
    with pytest.raises(lsdg.LsdgError):
        lsdg.calibration_load_xml("/nonexistent/calib.xml")


def test_reference_sample_calibration_parses():
    """The reference's own sample calibration (d2_camera.xml at the reference's top level, named by
    d2_ex1605l3_one.conf), kept as a fixture in tests/golden/."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "d2_camera.xml")
    c = lsdg.calibration_load_xml(path)
    assert c.model == T.CALIB_FRAME and (c.width, c.height) == (1920, 1080)
    assert (c.f, c.cx, c.cy, c.b2) == (1430.15016509976, -24.1342060175983, 17.5452248329602, -4.25145544487403)
    assert (c.k1, c.k2, c.p1, c.p2) == (-0.118322055927498, 0.293632083518507, 0.000330080086304322,
                                        0.00182154893322038)
    assert (c.b1, c.k3, c.k4) == (0.0, 0.0, 0.0)


def test_map_matches_numpy_restatement():
    c = calib_frame()
    K = default_K(c)
    got = lsdo.undistort_map(c, 640, 480, K)
    assert got.tobytes() == numpy_map(c, 640, 480, K).tobytes()
    K2 = T.Intrinsics(400.0, 410.0, 300.5, 250.25)
    assert lsdo.undistort_map(c, 600, 500, K2).tobytes() == numpy_map(c, 600, 500, K2).tobytes()


def test_pinhole_default_camera_is_identity():
    c = T.Calibration()
    c.model, c.width, c.height, c.f, c.cx, c.cy = T.CALIB_PINHOLE, 64, 48, 50.0, 1.5, -2.25
    c.k1 = 0.3  # ignored by the pinhole model
    m = lsdo.undistort_map(c, 64, 48, default_K(c))
    np.testing.assert_array_equal(m[..., 0], np.arange(64, dtype=np.float32)[None, :].repeat(48, 0))
    np.testing.assert_array_equal(m[..., 1], np.arange(48, dtype=np.float32)[:, None].repeat(64, 1))
    raw = np.random.default_rng(0).integers(0, 256, (48, 64)).astype(np.uint8)
    np.testing.assert_array_equal(lsdo.undistort(raw, m), raw)


def test_radial_displacement_on_axis():
    """On the row next to the principal point (y = -0.005) with only k1, the source is
    u = w/2 + cx + f x (1 + k1 (x^2 + y^2))."""
    c = T.Calibration()
    c.model, c.width, c.height, c.f, c.k1 = T.CALIB_FRAME, 200, 100, 100.0, -0.2
    K = T.Intrinsics(100.0, 100.0, 99.5, 49.5)
    m = lsdo.undistort_map(c, 200, 100, K)
    x = (np.arange(200) - 99.5) / 100.0
    np.testing.assert_allclose(m[49, :, 0] + 0.5, 100.0 + 100.0 * x * (1 - 0.2 * (x * x + 0.005 ** 2)), atol=1e-4)
    # barrel (k1 < 0): image corners sample from inside the raw frame
    assert 0 < m[0, 0, 0] and 0 < m[0, 0, 1]


def test_remap_of_smooth_pattern():
    c = calib_frame()
    m = lsdo.undistort_map(c, 640, 480, default_K(c))
    yy, xx = np.mgrid[0:480, 0:640].astype(np.float64)
    g = lambda u, v: 127.5 + 100 * np.sin(u / 23.0) * np.cos(v / 17.0)
    raw = np.clip(np.rint(g(xx, yy)), 0, 255).astype(np.uint8)
    out = lsdo.undistort(raw, m)
    inside = (m[..., 0] > 2) & (m[..., 1] > 2) & (m[..., 0] < 637) & (m[..., 1] < 477)
    ref = g(m[..., 0].astype(np.float64), m[..., 1].astype(np.float64))
    assert inside.mean() > 0.9
    assert np.abs(out[inside] - ref[inside]).max() < 3.0
    assert np.all(out[~((m[..., 0] >= 0) & (m[..., 1] >= 0) & (m[..., 0] <= 639) & (m[..., 1] <= 479))] == 0)
