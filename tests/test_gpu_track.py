"""GPU parity of the direct-alignment path (through the C-ABI) against the CPU oracle.

Bars: pyramids, depth pyramids and reference points bit-exact (integer-like float work with the
same operation order); normal-equation sums within 1e-4 relative (the summation order differs;
the oracle compensates every sum, the kernel its merges and the per-thread gradient and energy
sums, its per-thread Hessian sums run over a few dozen points); final poses within 1e-4 rad /
1e-4 m of the FP64 oracle and 1e-5 of the float oracle."""
import numpy as np
import pytest

import lsdg
import lsdg_types as T
import lsdo
import synth

pytestmark = pytest.mark.gpu

POSE_TOL_FP64 = 1e-4   # rad and m, against the FP64 oracle
POSE_TOL_F32 = 1e-5    # against the float oracle


def _frames(ctx, p):
    kf = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.ref_image).set_depth(p.ref_idepth, p.ref_idepth_var)
    fr = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.new_image)
    return kf, fr


@pytest.mark.parametrize("size", [(640, 480), (320, 240), (1280, 960)])
def test_pyramid_bit_exact(ctx, size):
    p = synth.tracking_pair(3, *size)
    f = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.new_image)
    ref = lsdo.pyramid(p.new_image, 5)
    for l in range(5):
        np.testing.assert_array_equal(f.level(l), ref[l])


def test_u8_upload_equals_float_upload(ctx):
    rng = np.random.default_rng(5)
    img8 = rng.integers(0, 256, (240, 320), dtype=np.uint8)
    k = synth.Intrinsics.for_size(320, 240)
    a = lsdg.Frame(ctx, 320, 240, k).upload(img8)
    b = lsdg.Frame(ctx, 320, 240, k).upload(img8.astype(np.float32))
    for l in range(5):
        np.testing.assert_array_equal(a.level(l), b.level(l))


def test_depth_pyramid_and_points_bit_exact(ctx, pair0):
    kf, _ = _frames(ctx, pair0)
    D, V, P, PV = lsdo.keyframe(pair0.ref_image, pair0.ref_idepth, pair0.ref_idepth_var, pair0.intr, 5)
    for l in range(5):
        d, v = kf.depth(l)
        np.testing.assert_array_equal(d, D[l])
        np.testing.assert_array_equal(v, V[l])
        xyzi, pv = kf.points(l)
        np.testing.assert_array_equal(xyzi, P[l])
        np.testing.assert_array_equal(pv, PV[l])


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
def test_normal_equations_match_oracle(ctx, pair0, level):
    kf, fr = _frames(ctx, pair0)
    rng = np.random.default_rng(level)
    T0 = synth.pose_mul(synth.random_motion(rng, (0.2, 0.5), (0.002, 0.01)), synth.pose_inv(pair0.frame_to_ref))
    got = lsdg.se3_normal_equations(ctx, kf, fr, level, T0)
    ref = lsdo.se3_normal_equations(pair0, T0, level)
    # the tracker is built with FMA contraction: a point within an ulp of the image margin may be
    # counted differently, everything else agrees to the summation-order level
    assert np.all(np.abs(got[28:32] - ref[28:32]) <= 2), (got[28:32], ref[28:32])
    scale = np.abs(ref[:27]).max()
    np.testing.assert_allclose(got[:27], ref[:27], rtol=1e-4, atol=2e-5 * scale)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_track_frame_matches_oracle(ctx, pairs4, seed):
    p = pairs4[seed]
    kf, fr = _frames(ctx, p)
    tracker = lsdg.SE3Tracker(ctx)
    T_gpu, st = tracker.trackFrame(kf, fr)
    rc, T_f, st_f = lsdo.track_se3(p)
    rcd, T_d, st_d = lsdo.track_se3(p, double=True)
    a_f, d_f = synth.pose_error(T_gpu, T_f)
    a_d, d_d = synth.pose_error(T_gpu, T_d)
    assert a_d <= POSE_TOL_FP64 and d_d <= POSE_TOL_FP64, (a_d, d_d)
    assert a_f <= POSE_TOL_F32 and d_f <= POSE_TOL_F32, (a_f, d_f)
    assert st.status == st_f.status == T.OK
    assert st.n_points == st_f.n_points
    assert abs(st.n_valid - st_f.n_valid) <= 5
    assert abs(st.total_passes - st_f.total_passes) <= 4, (list(st.passes), list(st_f.passes))


def test_track_frame_without_depth_points_is_lost(ctx, small_pair):
    kf = lsdg.Frame(ctx, small_pair.w, small_pair.h, small_pair.intr).upload(small_pair.ref_image)
    kf.set_depth(np.full_like(small_pair.ref_idepth, -1.0), small_pair.ref_idepth_var)
    fr = lsdg.Frame(ctx, small_pair.w, small_pair.h, small_pair.intr).upload(small_pair.new_image)
    T_gpu, st = lsdg.SE3Tracker(ctx).trackFrame(kf, fr)
    assert st.status == T.TRACKING_LOST
    assert st.total_passes == 0
    np.testing.assert_allclose(T_gpu, np.eye(3, 4))


def test_invalid_sizes_rejected(ctx):
    with pytest.raises(lsdg.LsdgError) as e:
        lsdg.Frame(ctx, 650, 480, synth.Intrinsics.for_size(640, 480))
    assert e.value.status == T.INVALID_ARG
    with pytest.raises(lsdg.LsdgError):
        lsdg.Batch(ctx, [], [], [])


def _mixed_pairs():
    sizes = [(320, 240)] * 3 + [(640, 480)] * 4 + [(1280, 960)] * 2
    return [synth.tracking_pair(100 + i, w, h) for i, (w, h) in enumerate(sizes)]


def test_batch_build_points_bit_exact(ctx):
    """The batch's one-launch build (pyramids, then each band's points at offsets found by a look-back
    over the bands before it) gives every keyframe's points bit for bit, mixed sizes, every level;
    again after a graph replay."""
    pairs = _mixed_pairs()
    b = lsdg.Batch(ctx, [p.w for p in pairs], [p.h for p in pairs], [p.intr for p in pairs])
    ri, rd, rv, ni = lsdg.pack_pairs(pairs)
    init = np.stack([np.eye(3, 4)] * len(pairs))
    for _ in range(2):
        b.track(ri, rd, rv, ni, init)
        for i in (0, 3, 7, 8):
            p = pairs[i]
            _, _, P, PV = lsdo.keyframe(p.ref_image, p.ref_idepth, p.ref_idepth_var, p.intr, 5)
            for l in range(5):
                xyzi, pv = b.points(i, l)
                np.testing.assert_array_equal(xyzi, P[l])
                np.testing.assert_array_equal(pv, PV[l])
    b.close()


def test_build_wait_that_runs_out_is_reported(ctx):
    """A band whose predecessor never publishes its counts (the test hook withholds band 0's) waits
    until its limit; the step reports TIMEOUT, nothing faults, and the next step is correct."""
    pairs = [synth.tracking_pair(600 + i, 320, 240) for i in range(2)]
    ri, rd, rv, ni = [np.ascontiguousarray(a) for a in lsdg.pack_pairs(pairs)]
    init = np.stack([np.eye(3, 4)] * 2)
    ref = lsdg.Batch(ctx, [320] * 2, [240] * 2, [p.intr for p in pairs])
    want, _ = ref.track(ri, rd, rv, ni, init)
    ref.close()
    b = lsdg.Batch(ctx, [320] * 2, [240] * 2, [p.intr for p in pairs])
    b.test_withhold(1)
    with pytest.raises(lsdg.LsdgError) as e:
        b.track(ri, rd, rv, ni, init)
    assert e.value.status == T.TIMEOUT
    b.test_withhold(-1)
    got, st = b.track(ri, rd, rv, ni, init)
    np.testing.assert_array_equal(got, want)
    assert all(s.status == T.OK for s in st)
    b.close()


def test_batch_matches_oracle_per_pair(ctx):
    pairs = _mixed_pairs()
    b = lsdg.Batch(ctx, [p.w for p in pairs], [p.h for p in pairs], [p.intr for p in pairs])
    ri, rd, rv, ni = lsdg.pack_pairs(pairs)
    init = np.stack([np.eye(3, 4)] * len(pairs))
    out, stats = b.track(ri, rd, rv, ni, init)
    for i, p in enumerate(pairs):
        rcd, T_d, _ = lsdo.track_se3(p, double=True)
        a, d = synth.pose_error(out[i], T_d)
        assert a <= POSE_TOL_FP64 and d <= POSE_TOL_FP64, (i, p.w, a, d)
        assert stats[i].status == T.OK
    # graph replay is deterministic and matches the first run
    out2, stats2 = b.track(ri, rd, rv, ni, init)
    np.testing.assert_array_equal(out, out2)
    shape = b.shape()
    assert shape["threads"] in (128, 256, 512) and shape["cluster"] in (2, 4, 8, 16)
    passes, pass_bytes, unique = b.work()
    assert passes == sum(s.total_passes for s in stats2)


def test_pipelined_batch_equals_synchronous(ctx):
    """submit/collect: two input sets alternating over the two slots give, in submission order,
    the synchronous results bit for bit; the synchronous calls refuse while steps are in flight."""
    sets = [[synth.tracking_pair(300 + 10 * k + i, 320, 240) for i in range(4)] for k in range(2)]
    intr = [p.intr for p in sets[0]]
    b = lsdg.Batch(ctx, [320] * 4, [240] * 4, intr)
    init = np.stack([np.eye(3, 4)] * 4)
    packed = [[np.ascontiguousarray(a) for a in lsdg.pack_pairs(s)] for s in sets]
    ref = [b.track(*packed[k], init)[0] for k in range(2)]
    order = [0, 1, 0, 1, 1]
    got = []
    b.submit(*packed[order[0]], init)
    for k in order[1:]:
        b.submit(*packed[k], init)
        with pytest.raises(lsdg.LsdgError):
            b.submit(*packed[k], init)        # a third step in flight
        with pytest.raises(lsdg.LsdgError):
            b.run()                           # synchronous form refuses meanwhile
        got.append(b.collect()[0])
    got.append(b.collect()[0])
    for k, g in zip(order, got):
        np.testing.assert_array_equal(g, ref[k])
    with pytest.raises(lsdg.LsdgError):
        b.collect()                           # nothing left
    np.testing.assert_array_equal(b.track(*packed[1], init)[0], ref[1])
    b.close()


def test_pipelined_u8_images_equal_float(ctx):
    """submit_u8 (8-bit images, widened to float on the device behind the copy) gives the float
    results bit for bit when the float images hold the same byte values, on the first step (graph
    capture) and on a replay."""
    pairs = [synth.tracking_pair(400 + i, 320, 240) for i in range(3)]
    b = lsdg.Batch(ctx, [320] * 3, [240] * 3, [p.intr for p in pairs])
    init = np.stack([np.eye(3, 4)] * 3)
    ri, rd, rv, ni = [np.ascontiguousarray(a) for a in lsdg.pack_pairs(pairs)]
    ri8 = np.clip(np.rint(ri), 0, 255).astype(np.uint8)
    ni8 = np.clip(np.rint(ni), 0, 255).astype(np.uint8)
    ref, ref_st = b.track(ri8.astype(np.float32), rd, rv, ni8.astype(np.float32), init)
    for _ in range(3):
        b.submit_u8(ri8, rd, rv, ni8, init)
        out, st = b.collect()
        np.testing.assert_array_equal(out, ref)
        assert [s.n_good for s in st] == [s.n_good for s in ref_st]
    with pytest.raises(AssertionError):
        b.submit_u8(ri, rd, rv, ni8, init)       # float images refused by the binding
    b.close()


def test_batch_with_lost_pair(ctx):
    pairs = [synth.tracking_pair(200, 320, 240), synth.tracking_pair(201, 320, 240)]
    pairs[1].ref_idepth = np.full_like(pairs[1].ref_idepth, -1.0)
    b = lsdg.Batch(ctx, [p.w for p in pairs], [p.h for p in pairs], [p.intr for p in pairs])
    out, stats = b.track(*lsdg.pack_pairs(pairs), np.stack([np.eye(3, 4)] * 2))
    assert stats[0].status == T.OK
    assert stats[1].status == T.TRACKING_LOST and stats[1].total_passes == 0


def test_launch_counter_counts_kernels(ctx, small_pair):
    n0 = ctx.launch_count()
    kf, fr = _frames(ctx, small_pair)
    # per image: band pyramid + gradients; depth: band pass + scan + scatter
    assert ctx.launch_count() - n0 == 2 + 2 + 3
