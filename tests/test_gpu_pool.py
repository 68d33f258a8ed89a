"""The pool plan of the batched SE3 tracker (track.cu, pool_kernel), pinned through
LSDG_TRACK_POOL so that it is tested whatever the autotuner picks: every pair of a mixed batch
within 1e-4 rad / 1e-4 m of the FP64 oracle, the pass counts and statuses of the float oracle, and
results independent of which CTA took which chunk (graph replays bit-identical), for several
shapes and chunk sizes."""
import os

import numpy as np
import pytest

import lsdo
import synth

pytestmark = pytest.mark.gpu

POSE_TOL = 1e-4


def _mixed():
    sizes = [(320, 240)] * 3 + [(640, 480)] * 4 + [(1280, 960)] * 2
    return synth.generate(synth.camera_pair, [(300 + i, w, h) for i, (w, h) in enumerate(sizes)],
                          min(9, os.cpu_count() or 4))


@pytest.fixture(scope="module")
def mixed():
    return _mixed()


def _pool_batch(pairs, pin):
    import lsdg
    os.environ["LSDG_TRACK_POOL"] = pin
    try:
        ctx = lsdg.Context()  # a fresh context: the plan is tuned (here: pinned) per context
        b = lsdg.Batch(ctx, [p.w for p in pairs], [p.h for p in pairs], [p.intr for p in pairs])
        b.load(*lsdg.pack_pairs(pairs), np.stack([np.eye(3, 4)] * len(pairs)))
        b.run()
    finally:
        del os.environ["LSDG_TRACK_POOL"]
    return ctx, b


@pytest.mark.parametrize("pin", ["256,2,2048", "512,1,4096", "128,4,2048"])
def test_pool_plan_vs_fp64_and_replays(mixed, pin):
    ctx, b = _pool_batch(mixed, pin)
    try:
        shape = b.shape()
        assert shape.get("plan") == "pool", shape
        assert shape["chunk_points"] == int(pin.split(",")[2])
        out, stats = b.read()
        ref, ref_stats = lsdo.track_batch(mixed, double=True)
        _, f_stats = lsdo.track_batch(mixed)
        for i in range(len(mixed)):
            ang, dist = synth.pose_error(out[i], ref[i])
            assert ang <= POSE_TOL and dist <= POSE_TOL, (i, ang, dist)
            assert stats[i].status == ref_stats[i].status
            assert abs(stats[i].total_passes - f_stats[i].total_passes) <= 4, (i, list(stats[i].passes),
                                                                               list(f_stats[i].passes))
        # which CTA takes which chunk changes from run to run; the partials merge in chunk order
        for _ in range(3):
            b.run()
            again, _ = b.read()
            np.testing.assert_array_equal(again, out)
    finally:
        b.close()
        ctx.close()


def test_pool_pair_without_points_is_lost(mixed):
    """A pair whose keyframe has no depth finishes in the set-up kernel (TRACKING_LOST, identity
    pose) while the other pairs of the batch track normally."""
    import lsdg_types as T
    pairs = [mixed[0], mixed[1]]
    empty = synth.camera_pair(301, 320, 240)
    empty.ref_idepth = np.full_like(empty.ref_idepth, -1.0)
    pairs = [pairs[0], empty, pairs[1]]
    ctx, b = _pool_batch(pairs, "256,2,2048")
    try:
        out, stats = b.read()
        assert stats[1].status == T.TRACKING_LOST and stats[1].total_passes == 0
        np.testing.assert_allclose(out[1], np.eye(3, 4))
        ref, _ = lsdo.track_batch([pairs[0], pairs[2]], double=True)
        for i, j in ((0, 0), (2, 1)):
            ang, dist = synth.pose_error(out[i], ref[j])
            assert ang <= POSE_TOL and dist <= POSE_TOL
    finally:
        b.close()
        ctx.close()
