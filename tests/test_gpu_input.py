"""GPU parity of the input step (raw 8-bit frame -> undistorted frame pyramid) through the C-ABI,
bit for bit against the CPU oracle."""
import numpy as np
import pytest

import lsdo
import lsdg_types as T
from test_oracle_input import calib_frame, default_K

pytestmark = pytest.mark.gpu


def test_undistorted_upload_matches_oracle(ctx):
    import lsdg
    c = calib_frame()
    u = lsdg.Undistorter(ctx, c)
    w, h, K = u.camera()
    assert (w, h) == (640, 480)
    Kd = default_K(c)
    assert (K.fx, K.fy, K.cx, K.cy) == (Kd.fx, Kd.fy, Kd.cx, Kd.cy)
    raw = np.random.default_rng(3).integers(0, 256, (480, 640)).astype(np.uint8)
    raw = np.ascontiguousarray(np.clip(raw.astype(np.int32) // 2 + 64, 0, 255).astype(np.uint8))
    f = lsdg.Frame(ctx, w, h, K)
    u.upload(f, raw)
    ref = lsdo.undistort(raw, lsdo.undistort_map(c, w, h, Kd))
    np.testing.assert_array_equal(u.last_image(), ref)
    np.testing.assert_array_equal(f.level(0)[..., 0], ref.astype(np.float32))
    np.testing.assert_array_equal(f.level(3), lsdo.pyramid(ref.astype(np.float32), 5)[3])
    u.close()


def test_custom_output_camera_and_errors(ctx):
    import lsdg
    c = calib_frame()
    K2 = T.Intrinsics(400.0, 400.0, 159.5, 119.5)
    u = lsdg.Undistorter(ctx, c, 320, 240, K2)
    raw = np.tile(np.arange(640, dtype=np.uint8)[None, :] // 3, (480, 1))
    f = lsdg.Frame(ctx, 320, 240, K2)
    u.upload(f, raw)
    ref = lsdo.undistort(raw, lsdo.undistort_map(c, 320, 240, K2))
    np.testing.assert_array_equal(u.last_image(), ref)
    wrong = lsdg.Frame(ctx, 640, 480, K2)
    with pytest.raises(lsdg.LsdgError):
        u.upload(wrong, raw)
    bad = T.Calibration()
    bad.model, bad.width, bad.height, bad.f = 7, 640, 480, 500.0
    with pytest.raises(lsdg.LsdgError):
        lsdg.Undistorter(ctx, bad)
    u.close()
