"""A short full-system run on the GPU (sequence.py over the C-ABI): 240 frames of the synthetic
room at 320x240 are tracked, mapped, turned into keyframes with batched Sim3 constraint search and a
pose graph; the trajectory stays within a few percent of the path length of the ground truth."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


def test_room_sequence_runs_end_to_end(ctx):
    import sequence
    seq, frames = synth.room_sequence(0, 240, 320, 240, workers=1)
    res = sequence.run(ctx, seq, frames)
    assert res["frames"] == 240 and res["non_finite_frames"] == 0
    assert res["lost_frames"] <= 5
    assert res["keyframes"] >= 15 and res["sim3_edges"] >= res["keyframes"]
    assert res["ate_over_path"] < 0.05, res
    assert 0.85 < res["alignment_scale"] < 1.15, res
