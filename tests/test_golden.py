"""The oracle (CPU) and the library (GPU) reproduce the frozen golden fixtures of tests/golden/."""
import json
import os
import sys

import numpy as np
import pytest

import lsdo

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden as G  # noqa: E402


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden_small.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def inputs():
    return G.load_inputs()


def test_oracle_reproduces_golden(golden, inputs):
    got = G.oracle_outputs(*inputs)
    for k in ("pyramid_sha", "points_sha", "points_count", "track_status", "track_passes", "depth_update_sha",
              "depth_propagate_sha", "depth_valid_after_update"):
        assert got[k] == golden[k], k
    np.testing.assert_allclose(got["track_pose"], golden["track_pose"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got["normal_equations_level1"], golden["normal_equations_level1"], rtol=1e-12)


@pytest.mark.gpu
def test_library_reproduces_golden(golden, inputs, ctx):
    import lsdg
    import synth
    p, s = inputs
    f = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.new_image)
    assert [G.sha(f.level(l)) for l in range(5)] == golden["pyramid_sha"]
    kf = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.ref_image).set_depth(p.ref_idepth, p.ref_idepth_var)
    assert [G.sha(kf.points(l)[0]) for l in range(5)] == golden["points_sha"]
    T, st = lsdg.SE3Tracker(ctx).trackFrame(kf, f)
    a, t = synth.pose_error(T, np.array(golden["track_pose"]).reshape(3, 4))
    assert a < 1e-5 and t < 1e-5
    dm = lsdg.DepthMap(ctx, s.w, s.h, s.intr).set_keyframe(s.key_image, s.init_idepth, s.init_var)
    dm.updateKeyframe(s.ref_images, [lsdo._inv(T_) for T_ in s.ref_frame_to_key])
    assert {k: G.sha(v) for k, v in dm.get().items()} == golden["depth_update_sha"]
    dm.createKeyFrame(s.next_image, lsdo._inv(s.next_to_key))
    assert {k: G.sha(v) for k, v in dm.get().items()} == golden["depth_propagate_sha"]
