"""Accuracy of the benchmark's own workloads against the FP64 oracle, through the C-ABI.

The tracker solves its LM systems in float on Jacobi-scaled normal equations and sums the Hessian
entries per thread without compensation; these tests show what that costs on the exact inputs the
benchmark times: every pair of the 64-pair 640x480 headline batch (seeds 0..63), of the 64-pair
mixed batch (20 x 320x240, 32 x 640x480, 12 x 1280x960, seeds 5000 + i) and of the 10-candidate
Sim3 constraint batch (seeds 2000 + i) must end within 1e-4 rad / 1e-4 m (Sim3: and 1e-4 of the
scale) of the FP64 oracle run on the same 8-bit inputs."""
import os

import numpy as np
import pytest

import lsdo
import synth

pytestmark = pytest.mark.gpu

POSE_TOL = 1e-4


def _workers():
    return min(16, os.cpu_count() or 4)


@pytest.fixture(scope="module")
def headline():
    return synth.generate(synth.camera_pair, [(i, 640, 480) for i in range(synth.HEADLINE_PAIRS)], _workers())


@pytest.fixture(scope="module")
def mixed():
    specs = [(synth.MIXED_SEED0 + i, w, h) for i, (w, h) in enumerate(synth.MIXED_SIZES)]
    return synth.generate(synth.camera_pair, specs, _workers())


def _track_batch(ctx, pairs):
    import lsdg
    b = lsdg.Batch(ctx, [p.w for p in pairs], [p.h for p in pairs], [p.intr for p in pairs])
    try:
        out, stats = b.track(*lsdg.pack_pairs(pairs), np.stack([np.eye(3, 4)] * len(pairs)))
    finally:
        b.close()
    return out, stats


def _assert_vs_fp64(pairs, out, stats):
    ref, ref_stats = lsdo.track_batch(pairs, threads=_workers(), double=True)
    errs = np.array([synth.pose_error(out[i], ref[i]) for i in range(len(pairs))])
    worst = int(np.argmax(errs.max(axis=1)))
    assert errs[:, 0].max() <= POSE_TOL and errs[:, 1].max() <= POSE_TOL, (worst, errs[worst])
    assert all(s.status == r.status for s, r in zip(stats, ref_stats))
    return errs


def test_headline_batch_vs_fp64(ctx, headline):
    out, stats = _track_batch(ctx, headline)
    _assert_vs_fp64(headline, out, stats)


def test_mixed_batch_vs_fp64(ctx, mixed):
    out, stats = _track_batch(ctx, mixed)
    _assert_vs_fp64(mixed, out, stats)


def test_sim3_constraint_batch_vs_fp64(ctx):
    import lsdg
    sps = synth.generate(synth.sim3_pair, [(synth.SIM3_SEED0 + i, 640, 480) for i in range(synth.SIM3_CANDIDATES)],
                         _workers())
    b = lsdg.Batch(ctx, [q.w for q in sps], [q.h for q in sps], [q.intr for q in sps], sim3=True)
    try:
        init = np.tile(np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]]), (len(sps), 1))
        b.load_sim3(*lsdg.pack_sim3_pairs(sps), init)
        b.run()
        out, stats = b.read()
    finally:
        b.close()
    for i, q in enumerate(sps):
        rc, o, _ = lsdo.track_sim3(q, double=True)
        assert stats[i].status == rc == 0
        ang, dist, ds = lsdo.sim3_error(out[i], o)
        assert ang <= POSE_TOL and dist <= POSE_TOL and ds <= POSE_TOL, (i, ang, dist, ds)
