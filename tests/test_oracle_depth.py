"""CPU tests of the depth-filter oracle: it recovers the synthetic scene's inverse depth, the float
and FP64 restatements agree on the flags, and the stages behave as specified."""
import numpy as np
import pytest

import lsdo
import synth


@pytest.fixture(scope="module")
def seq():
    return synth.depth_sequence(0, 320, 240)


def test_update_recovers_scene_depth(seq):
    upd, prop = lsdo.depth_pipeline(seq, propagate=False)
    good = (upd["validity"] > 0) & (upd["var"] < 0.01)
    assert good.sum() > 5000
    rel = np.abs(upd["idepth"][good] - seq.key_true_idepth[good]) / seq.key_true_idepth[good]
    assert np.median(rel) < 0.05, np.median(rel)


def test_float_and_fp64_oracles_agree_on_flags(seq):
    f, _ = lsdo.depth_pipeline(seq, propagate=False)
    d, _ = lsdo.depth_pipeline(seq, propagate=False, double=True)
    assert np.mean(f["validity"] == d["validity"]) >= 0.999
    assert np.mean(f["blacklist"] == d["blacklist"]) >= 0.999
    both = (f["validity"] > 0) & (d["validity"] > 0) & (f["var"] < 0.01)
    rel = np.abs(f["idepth"][both] - d["idepth"][both]) / d["idepth"][both]
    assert np.mean(rel < 1e-3) >= 0.99


def test_observe_without_regularize_keeps_unobserved_pixels(seq):
    upd, _ = lsdo.depth_pipeline(seq, propagate=False, regularize=False, n_refs=1)
    gx, gy = synth.central_gradient(seq.key_image.astype(np.float64))
    flat = (gx * gx + gy * gy) < 25.0  # below min_grad: never observed
    np.testing.assert_array_equal(upd["idepth"][flat], seq.init_idepth[flat])
    np.testing.assert_array_equal(upd["blacklist"][flat], 0)


def test_propagation_moves_hypotheses_to_new_keyframe(seq):
    upd, prop = lsdo.depth_pipeline(seq)
    assert (prop["validity"] > 0).sum() > 0.3 * (upd["validity"] > 0).sum()
    # propagated variance never shrinks below the prediction noise
    v = prop["var"][prop["validity"] > 0]
    assert np.all(v >= lsdo.default_params().prediction_var * 0.999)


def test_multithreaded_update_is_identical(seq):
    a, _ = lsdo.depth_pipeline(seq, propagate=False, threads=1)
    b, _ = lsdo.depth_pipeline(seq, propagate=False, threads=4)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_no_hypotheses_stay_empty(seq):
    none = np.full((seq.h, seq.w), -1.0, np.float32)
    upd, _ = lsdo.depth_pipeline(seq, propagate=False, init_idepth=none)
    # pixels with gradient get new hypotheses from the first successful observation
    assert (upd["validity"] > 0).sum() > 1000
