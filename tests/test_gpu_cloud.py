"""GPU parity of the keyframe point cloud (Keyframe::computeVbo's filter and back-projection,
publishKeyframe's export) through the C-ABI, bit for bit against the CPU oracle and against the
reference's own computeVbo loop (the committed fixture of its outputs, and the loop compiled from
Keyframe.h where oracle/_ref is present)."""
import numpy as np
import pytest

import lsdo
import synth
from test_oracle_cloud import K, H, W, _edge_keyframes, random_keyframe, reference_cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("scale", [1.0, 12.0])
def test_cloud_build_matches_oracle(ctx, seed, scale):
    import lsdg
    pts = random_keyframe(seed)
    got = lsdg.cloud_build(ctx, pts, W, H, *K, scale=scale)
    ref = lsdo.cloud_build(pts, W, H, *K, scale=scale)
    assert len(got) == len(ref) > 100
    assert got.tobytes() == ref.tobytes()


def test_cloud_build_matches_reference_fixture(ctx):
    import lsdg
    for pts, w, h, fx, fy, cx, cy, scale, v in reference_cases():
        got = lsdg.cloud_build(ctx, pts.reshape(-1), w, h, fx, fy, cx, cy, scale=scale)
        assert len(got) == len(v) > 500
        assert got.tobytes() == v.tobytes()


def test_cloud_build_matches_reference_code(ctx):
    import lsdg
    if lsdo.ref_lib() is None:
        pytest.skip("oracle/_ref not built: the reference tree is absent")
    cases = [(f"seed {s}", random_keyframe(s + 200, 160, 120), sc) for s in range(2) for sc in (0.5, 4.0)]
    for name, pts, scale in cases + list(_edge_keyframes()):
        h, w = pts.shape
        ref = lsdo.ref_compute_vbo(pts, w, h, *K, scale=scale)
        got = lsdg.cloud_build(ctx, pts.reshape(-1), w, h, *K, scale=scale)
        assert got.tobytes() == ref.tobytes(), name


def test_cloud_build_full_frame_and_params(ctx):
    import lsdg
    pts = random_keyframe(5, 640, 480)
    got = lsdg.cloud_build(ctx, pts, 640, 480, 500.0, 500.0, 320.0, 240.0)
    ref = lsdo.cloud_build(pts, 640, 480, 500.0, 500.0, 320.0, 240.0)
    assert got.tobytes() == ref.tobytes()
    p = lsdg.cloud_default_params()
    p.min_near_support = 5
    p.scaled_th = 5e-4
    got = lsdg.cloud_build(ctx, pts, 640, 480, 500.0, 500.0, 320.0, 240.0, params=p)
    ref = lsdo.cloud_build(pts, 640, 480, 500.0, 500.0, 320.0, 240.0, scaled_th=5e-4, min_near_support=5)
    assert got.tobytes() == ref.tobytes()
    empty = np.zeros(640 * 480, lsdg.POINT_DENSE)
    assert len(lsdg.cloud_build(ctx, empty, 640, 480, 500.0, 500.0, 320.0, 240.0)) == 0


def test_depthmap_export_and_device_cloud(ctx):
    """publishKeyframe's export of the depth map's keyframe, and the cloud built from it on the
    device into a caller-owned buffer, against the oracle applied to the exported points."""
    import torch

    import lsdg
    seq = synth.depth_sequence(3, 320, 240, n_refs=4)
    dm = lsdg.DepthMap(ctx, seq.w, seq.h, seq.intr).set_keyframe(seq.key_image, seq.init_idepth, seq.init_var)
    dm.updateKeyframe(seq.ref_images, [synth.pose_inv(T) for T in seq.ref_frame_to_key])
    st = dm.get()
    pts = dm.export_points()
    np.testing.assert_array_equal(pts["idepth"], st["idepth_smoothed"])
    np.testing.assert_array_equal(pts["idepth_var"], st["var_smoothed"])
    img = np.clip(seq.key_image, 0, 255).astype(np.float32)
    u8 = np.where(img >= 255, 255, np.floor(img)).astype(np.uint8)
    for k in range(4):
        np.testing.assert_array_equal(pts["color"][..., k], u8)
    buf = torch.empty(seq.w * seq.h * 4, dtype=torch.float32, device="cuda")
    # the reference's thresholds keep few points of a 4-frame map; relaxed ones keep thousands
    relaxed = lsdg.cloud_default_params()
    relaxed.scaled_th, relaxed.abs_th, relaxed.min_near_support = 1.0, 10.0, 5
    for scale, params, kw, least in ((1.0, None, {}, 0),
                                     (0.5, relaxed, dict(scaled_th=1.0, abs_th=10.0, min_near_support=5), 1000)):
        n = dm.cloud_to_device(buf.data_ptr(), scale=scale, params=params)
        torch.cuda.synchronize()
        got = np.frombuffer(buf[:4 * n].cpu().numpy().tobytes(), lsdg.CLOUD_VERTEX)
        ref = lsdo.cloud_build(pts, seq.w, seq.h, *seq.intr.as_tuple(), scale=scale, **kw)
        assert n == len(ref) and n >= least
        assert got.tobytes() == ref.tobytes()
    with pytest.raises(lsdg.LsdgError):
        dm.cloud_to_device(buf.data_ptr() + 4)  # not 16-byte aligned
    dm.close()
