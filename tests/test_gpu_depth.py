"""GPU parity of the depth filter (observeDepth / regularizeDepthMap / propagateDepth) through the
C-ABI against the CPU oracle.

Bars: every state plane bit-identical to the float oracle (same operation order, no FMA
contraction on either side); against the FP64 oracle the validity and blacklist flags agree on at
least 99.9 % of pixels and well-observed inverse depths agree within 1e-3 relative."""
import numpy as np
import pytest

import lsdg
import lsdg_types as T
import lsdo
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seq640():
    return synth.depth_sequence(0, 640, 480)


@pytest.fixture(scope="module")
def seq320():
    return synth.depth_sequence(3, 320, 240)


def _gpu_pipeline(ctx, seq, regularize=True, propagate=True, n_refs=None):
    n = len(seq.ref_images) if n_refs is None else n_refs
    dm = lsdg.DepthMap(ctx, seq.w, seq.h, seq.intr).set_keyframe(seq.key_image, seq.init_idepth, seq.init_var)
    dm.updateKeyframe(seq.ref_images[:n], [lsdo._inv(T_) for T_ in seq.ref_frame_to_key[:n]], regularize=regularize)
    upd = dm.get()
    prop = None
    if propagate:
        dm.createKeyFrame(seq.next_image, lsdo._inv(seq.next_to_key), regularize=regularize)
        prop = dm.get()
    dm.close()
    return upd, prop


def _assert_planes_equal(got, ref):
    for k in lsdo.DEPTH_PLANES:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.parametrize("n_refs", [1, 8])
def test_observe_bit_exact(ctx, seq320, n_refs):
    got, _ = _gpu_pipeline(ctx, seq320, regularize=False, propagate=False, n_refs=n_refs)
    ref, _ = lsdo.depth_pipeline(seq320, regularize=False, propagate=False, n_refs=n_refs)
    _assert_planes_equal(got, ref)


def test_update_regularize_propagate_bit_exact_640(ctx, seq640):
    got_u, got_p = _gpu_pipeline(ctx, seq640)
    ref_u, ref_p = lsdo.depth_pipeline(seq640)
    _assert_planes_equal(got_u, ref_u)
    _assert_planes_equal(got_p, ref_p)


def test_flags_and_idepth_vs_fp64_oracle(ctx, seq640):
    """Against the FP64 oracle: flags agree on >= 99.9 % of pixels, the observed inverse depths
    within 1e-3 relative on >= 99.9 % of the pixels holding one in both runs, and every pixel whose
    flags differ -- after the update and after the propagation into the next keyframe -- is
    explained by a decision at a float threshold boundary (tests/depth_flags.py)."""
    import depth_flags
    got_u, got_p = _gpu_pipeline(ctx, seq640)
    c, upd, prop = depth_flags.classify(seq640)
    for got, ref in ((got_u, c.upd_d), (got_p, c.prop_d)):
        assert np.mean(got["validity"] == ref["validity"]) >= 0.999
        assert np.mean(got["blacklist"] == ref["blacklist"]) >= 0.999
    moved = got_u["var"] != seq640.init_var
    both = (got_u["validity"] > 0) & (c.upd_d["validity"] > 0) & moved
    rel = np.abs(got_u["idepth"][both] - c.upd_d["idepth"][both]) / c.upd_d["idepth"][both]
    assert np.mean(rel <= 1e-3) >= 0.999, np.mean(rel <= 1e-3)
    # the GPU's disagreements are the float oracle's (its state is the float oracle's bit for bit)
    np.testing.assert_array_equal(depth_flags.flags_differ(got_u, c.upd_d), depth_flags.flags_differ(c.upd_f, c.upd_d))
    np.testing.assert_array_equal(depth_flags.flags_differ(got_p, c.prop_d), depth_flags.flags_differ(c.prop_f, c.prop_d))
    bad = [{k: v for k, v in r.items() if k != "via"} for r in upd + prop if not r["explained"]]
    assert not bad, bad


def test_depth_output_layout(ctx, seq320):
    """idepth <= 0 marks 'no depth' in the planes the viewer reads (Keyframe.h:95)."""
    got, _ = _gpu_pipeline(ctx, seq320, propagate=False)
    none = got["validity"] <= 0
    assert np.all(got["idepth"][none] == -1.0)
    assert got["idepth"].shape == (seq320.h, seq320.w) and got["idepth"].dtype == np.float32


def test_depth_argument_errors(ctx, seq320):
    dm = lsdg.DepthMap(ctx, seq320.w, seq320.h, seq320.intr)
    with pytest.raises(lsdg.LsdgError) as e:  # no keyframe yet
        dm.updateKeyframe(seq320.ref_images[:1], [np.eye(3, 4)])
    assert e.value.status == T.INVALID_ARG
    dm.set_keyframe(seq320.key_image, seq320.init_idepth, seq320.init_var)
    with pytest.raises(lsdg.LsdgError):
        dm.updateKeyframe(seq320.ref_images[:1] * 17, [np.eye(3, 4)] * 17)
    dm.close()


def test_u8_reference_frames_equal_float_path(ctx):
    """lsdg_depth_update_u8 (8-bit frames, converted on the device) gives the state of the float path
    on the same (quantised) frames, bit for bit."""
    import lsdg
    import synth
    seq = synth.depth_sequence(11, 320, 240, n_refs=4)
    q = [np.clip(np.rint(r), 0, 255).astype(np.uint8) for r in seq.ref_images]
    poses = [synth.pose_inv(T) for T in seq.ref_frame_to_key]
    a = lsdg.DepthMap(ctx, seq.w, seq.h, seq.intr).set_keyframe(seq.key_image, seq.init_idepth, seq.init_var)
    a.updateKeyframe([x.astype(np.float32) for x in q], poses)
    b = lsdg.DepthMap(ctx, seq.w, seq.h, seq.intr).set_keyframe(seq.key_image, seq.init_idepth, seq.init_var)
    b.updateKeyframe_u8(np.ascontiguousarray(np.stack(q)), poses)
    sa, sb = a.get(), b.get()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    part = b.get(planes=("idepth_smoothed", "var_smoothed"))
    assert set(part) == {"idepth_smoothed", "var_smoothed"}
    np.testing.assert_array_equal(part["idepth_smoothed"], sa["idepth_smoothed"])
    a.close()
    b.close()
