"""Full-system runs on the GPU through the library's SLAM loop (lsdg_slam over the C-ABI, driven
by sequence.py): frames of the synthetic room are tracked, mapped, turned into keyframes (or an
earlier keyframe is made current again) with batched two-way Sim3 constraint search and a Sim3 pose
graph; the trajectory stays within a few percent of the path length of the ground truth at 320x240
and 640x480 over 240 frames, and within 2 % over the full 1,000-frame sequence."""
import os

import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


def _check(res, n):
    assert res["frames"] == n and res["non_finite_frames"] == 0
    assert res["lost_frames"] <= 5, res
    assert res["keyframes"] >= 15 and res["sim3_edges"] >= res["keyframes"] - 1, res
    assert res["keyframe_graph_nodes"] == res["keyframes"]


def test_room_sequence_320x240(tmp_path):
    import sequence
    seq, frames = synth.room_sequence(0, 240, 320, 240, workers=min(8, os.cpu_count() or 2))
    res = sequence.run(seq, frames, pose_file=str(tmp_path / "pose.txt"))
    _check(res, 240)
    assert res["ate_over_path"] < 0.05, res
    assert res["ate_over_gt_spread"] < 0.35, res   # well below a trajectory collapsed to its mean
    assert 0.85 < res["alignment_scale"] < 1.15, res
    rows = (tmp_path / "pose.txt").read_text().splitlines()
    assert len(rows) == 240 and rows[0].startswith("0,") and all(len(r.split(",")) == 7 for r in rows)


def test_room_sequence_640x480():
    import sequence
    seq, frames = synth.room_sequence(0, 240, 640, 480, workers=min(16, os.cpu_count() or 2))
    res = sequence.run(seq, frames)
    _check(res, 240)
    assert res["ate_over_path"] < 0.05, res
    assert res["ate_over_gt_spread"] < 0.35, res


def test_room_sequence_1000_frames():
    """The full sequence of the benchmark (seed 0: 1,000 frames 640x480, the path driven 2.2 times):
    each keyframe is refined before it is left (its frames tracked again against its depth, the depth
    mapped again from the new poses), and on the second lap earlier keyframes are made current again,
    which closes the loop; ATE under 2 % of the path and under 0.15 of the ground truth's own spread
    (measured on the rooms of seeds 0-5: 0.11-0.84 % and 0.015-0.114), the map's scale within 25 %
    (monocular: the scale drifts; measured 0.99-1.12)."""
    import sequence
    seq, frames = synth.room_sequence(0, 1000, 640, 480, workers=min(16, os.cpu_count() or 2))
    res = sequence.run(seq, frames)
    assert res["frames"] == 1000 and res["non_finite_frames"] == 0
    assert res["lost_frames"] <= 5, res
    assert res["reactivations"] > 0, res
    assert res["ate_over_path"] < 0.02, res
    assert res["ate_over_gt_spread"] < 0.15, res
    assert 0.8 < res["alignment_scale"] < 1.25, res


def test_keyframe_depth_against_truth():
    """The loop's keyframe depth maps (lsdg_slam_keyframe_depth) over the first 60 frames at 640x480:
    median inverse depth within 3 % of the rendered truth and under 5 % of the pixels off by more
    than 20 % (measured: 1.003-1.007 and 0.7-2.2 %)."""
    import lsdg
    import sequence
    seq, frames = synth.room_sequence(0, 60, 640, 480, workers=min(16, os.cpu_count() or 2), keep_depths=True)
    sys_ = lsdg.SlamSystem(seq.w, seq.h, seq.intr)
    try:
        idepth, var = sequence.bootstrap_depth(seq, image=frames[0])
        sys_.bootstrap(0, frames[0], idepth, var)
        for k in range(1, 60):
            sys_.nextImage(k, frames[k])
        nk = sys_.stats()["keyframes"]
        assert nk >= 6
        for k in range(nk):
            fid, d, v = sys_.keyframe_depth(k)
            D = seq.depths[fid]
            ok = (d > 0) & np.isfinite(D) & (D > 0)
            assert ok.sum() > 50000, (k, int(ok.sum()))
            r = d[ok] * D[ok]
            assert abs(float(np.median(r)) - 1.0) < 0.03, (k, float(np.median(r)))
            assert float(np.mean(np.abs(r - 1.0) > 0.2)) < 0.05, k
    finally:
        sys_.close()


def test_inline_constraints_equal_worker_thread():
    """The constraint search on the worker thread (joined before each new keyframe) gives the
    trajectory of the same search run inline, bit for bit."""
    seq, frames = synth.room_sequence(1, 90, 320, 240, workers=min(8, os.cpu_count() or 2))
    out = []
    # one launch shape for every tracker call of both systems (the autotuner's pick could differ
    # between them, and with it the summation order)
    os.environ["LSDG_TRACK_SHAPE"] = "256,8,2"
    try:
        _run_both(seq, frames, out)
    finally:
        del os.environ["LSDG_TRACK_SHAPE"]
    np.testing.assert_array_equal(out[0], out[1])


def _run_both(seq, frames, out):
    import lsdg
    import sequence
    for inline in (0, 1):
        sp = lsdg.slam_default_params()
        sp.async_constraints = 1 - inline
        sys_ = lsdg.SlamSystem(seq.w, seq.h, seq.intr, slam_params=sp)
        idepth, var = sequence.bootstrap_depth(seq, image=frames[0])
        sys_.bootstrap(0, frames[0], idepth, var)
        for k in range(1, 90):
            sys_.nextImage(k, frames[k])
        sys_.finalize()
        out.append(sys_.poses())
        sys_.close()
