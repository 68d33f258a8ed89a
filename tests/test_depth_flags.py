"""Every validity / blacklist disagreement between the float depth filter and the FP64 oracle sits
at a float threshold boundary (CPU; the GPU depth kernels equal the float oracle bit for bit, which
test_gpu_depth.py checks, so this classifies the GPU's disagreements too).

Workloads: the keyframe update of synth.depth_sequence(0, 640, 480) -- 8 references on a 10 cm
arc, observe + regularise -- and the new keyframe it propagates into (propagate + regularise);
the same at 320x240 (seed 3).  The classifier (tests/depth_flags.py) walks both runs' decision
traces to the first decision they took differently and requires a threshold straddle within
2e-3 relative, a near-tie of an argmin, or a neighbour / source pixel whose own divergence is
explained the same way."""
import numpy as np
import pytest

import depth_flags
import lsdo
import synth


@pytest.fixture(scope="module")
def seq640():
    return synth.depth_sequence(0, 640, 480)


def _assert_all_explained(results):
    bad = [{k: v for k, v in r.items() if k != "via"} for r in results if not r["explained"]]
    assert not bad, bad


def test_update_and_propagation_disagreements_at_thresholds_640(seq640):
    c, upd, prop = depth_flags.classify(seq640)
    # the flags agree on at least 99.9 % of pixels, and every pixel that differs is explained
    for a, b in ((c.upd_f, c.upd_d), (c.prop_f, c.prop_d)):
        assert np.mean(~depth_flags.flags_differ(a, b)) >= 0.999
    assert len(upd) + len(prop) > 0  # the workload does exercise the classifier
    _assert_all_explained(upd)
    _assert_all_explained(prop)
    assert depth_flags.worst_margin(upd + prop) <= 2e-3


def test_disagreements_at_thresholds_320():
    _, upd, prop = depth_flags.classify(synth.depth_sequence(3, 320, 240))
    _assert_all_explained(upd)
    _assert_all_explained(prop)


def test_trace_records_in_execution_order(seq640):
    """A traced pixel's observe records start with the blacklist check of reference 0 and its
    gradient test; untraced pixels leave no record."""
    mask = np.zeros((4, seq640.h, seq640.w), bool)
    y, x = 240, 321
    mask[0, y, x] = True
    tr = lsdo.depth_trace(seq640, mask, propagate=False)
    assert len(tr) > 0 and np.all(tr["pixel"] == y * seq640.w + x) and np.all(tr["stage"] == 0)
    assert [int(tr["id"][0]), int(tr["id"][1])] == [depth_flags.D["BLLIMIT"], depth_flags.D["GRAD"]]
    assert np.all(np.diff(tr["ref"]) >= 0)


def test_classifier_rejects_a_planted_threshold_change(seq640):
    """A difference that is not rounding -- the FP64 run given a 2 % larger uniqueness ratio --
    leaves disagreements the classifier refuses to explain."""
    p = lsdo.default_params()
    q = lsdo.default_params()
    q.unique_ratio = p.unique_ratio * 1.02
    _, upd, prop = depth_flags.classify(seq640, params=p, params_fp64=q, propagate=False)
    assert sum(1 for r in upd if not r["explained"]) > 0
