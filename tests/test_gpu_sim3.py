"""GPU parity of Sim3 direct alignment (Sim3Tracker::trackFrameSim3) through the C-ABI against the
CPU oracle: the normal-equation record of one pass, the tracked similarity (rotation and translation
within 1e-4 rad / 1e-4 m and scale within 1e-4 of the FP64 oracle), the batched form, and the
argument checks."""
import numpy as np
import pytest

import lsdo
import synth

pytestmark = pytest.mark.gpu

_cache = {}


def spair(seed, w=640, h=480):
    key = (seed, w, h)
    if key not in _cache:
        _cache[key] = synth.sim3_pair(seed, w, h)
    return _cache[key]


def frames(ctx, sp):
    import lsdg
    ref = lsdg.Frame(ctx, sp.w, sp.h, sp.intr).upload(sp.ref_image).set_depth(sp.ref_idepth, sp.ref_idepth_var)
    cur = lsdg.Frame(ctx, sp.w, sp.h, sp.intr).upload(sp.new_image).set_depth(sp.new_idepth, sp.new_idepth_var)
    return ref, cur


def _true_ref_to_frame13(sp):
    s = sp.frame_to_ref13[12]
    M = np.concatenate([np.reshape(sp.frame_to_ref13[:9], (3, 3)) * s, np.reshape(sp.frame_to_ref13[9:12], (3, 1))], 1)
    A = np.linalg.inv(np.vstack([M, [0, 0, 0, 1]]))[:3]
    si = np.cbrt(np.linalg.det(A[:, :3]))
    return np.concatenate([(A[:, :3] / si).ravel(), A[:, 3], [si]])


@pytest.mark.parametrize("level", [0, 2, 4])
@pytest.mark.parametrize("at_truth", [False, True])
def test_sim3_normal_equations_match_oracle(ctx, level, at_truth):
    import lsdg
    sp = spair(0)
    ref, cur = frames(ctx, sp)
    T13 = _true_ref_to_frame13(sp) if at_truth else np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]])
    g = lsdg.sim3_normal_equations(ctx, ref, cur, level, T13)
    o = lsdo.sim3_normal_equations(sp, T13, level)
    # counts: a point whose projection is within rounding of the border may fall either side
    for i in range(36, 40):
        assert abs(g[i] - o[i]) <= 2, (i, g[i], o[i])
    # sums: float kernel vs float oracle.  The bilinear depth derivative jumps at pixel borders, so a
    # point that lands within rounding of one can move the record.  How far is measured, not assumed:
    # the oracle's own record under six pose perturbations of 1e-7 (rad, m) -- the size of the float
    # rounding the kernel's projections differ by -- spreads by up to 1.6e-3 of its scale at the
    # identity pose (every projection on a pixel centre) and 3e-5 at the true pose.  The kernel's
    # record must lie within 3x that spread plus 1e-4 of the scale.
    scale = np.abs(o[:36]).max()
    spread = _rounding_spread(sp, T13, level, o)
    np.testing.assert_allclose(g[:36], o[:36], rtol=0, atol=(3.0 * spread + 1e-4) * scale)


def _rotvec(w):
    th = np.linalg.norm(w)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def _rounding_spread(sp, T13, level, o):
    """Largest change of the oracle's Sim3 record (relative to its scale) under pose perturbations
    of 1e-7 rad / 1e-7 m."""
    rng = np.random.default_rng(level)
    scale = np.abs(o[:36]).max()
    out = 0.0
    for _ in range(6):
        d = np.array(T13, np.float64)
        d[:9] = (_rotvec(1e-7 * rng.normal(size=3)) @ d[:9].reshape(3, 3)).ravel()
        d[9:12] += 1e-7 * rng.normal(size=3)
        out = max(out, float(np.abs(lsdo.sim3_normal_equations(sp, d, level)[:36] - o[:36]).max() / scale))
    return out


def test_sim3_normal_equations_photometric_block_tight(ctx):
    """With the inverse-depth term switched off the record is smooth: float-level agreement."""
    import lsdg
    sp = spair(0)
    p = lsdg.default_params()
    p.sim3_depth_weight = 0.0
    c2 = lsdg.Context(p)
    try:
        ref, cur = frames(c2, sp)
        T13 = _true_ref_to_frame13(sp)
        for level in (0, 3):
            g = lsdg.sim3_normal_equations(c2, ref, cur, level, T13)
            o = lsdo.sim3_normal_equations(sp, T13, level, params=p)
            scale = np.abs(o[:36]).max()
            np.testing.assert_allclose(g[:36], o[:36], rtol=0, atol=1e-4 * scale)
    finally:
        c2.close()


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_track_sim3_matches_fp64_oracle(ctx, seed):
    import lsdg
    sp = spair(seed)
    ref, cur = frames(ctx, sp)
    (Tg, sg), st = lsdg.Sim3Tracker(ctx).trackFrameSim3(ref, cur)
    assert st.status == 0
    rc, o, ost = lsdo.track_sim3(sp, double=True)
    assert rc == 0
    got = lsdg._pose13((Tg, sg))
    ang, dist, ds = lsdo.sim3_error(got, o)
    assert ang < 1e-4 and dist < 1e-4 and ds < 1e-4, (ang, dist, ds)
    # and both recover the synthetic similarity to the accuracy the 5 % depth noise allows
    ang, dist, ds = lsdo.sim3_error(got, sp.frame_to_ref13)
    assert ang < 5e-3 and dist < 2e-2 and ds < 5e-2, (ang, dist, ds)


def test_track_sim3_from_truth_stays(ctx):
    import lsdg
    sp = spair(1)
    ref, cur = frames(ctx, sp)
    (Tg, sg), st = lsdg.Sim3Tracker(ctx).trackFrameSim3(ref, cur, (np.concatenate(
        [np.reshape(sp.frame_to_ref13[:9], (3, 3)), np.reshape(sp.frame_to_ref13[9:12], (3, 1))], 1),
        sp.frame_to_ref13[12]))
    rc, o, _ = lsdo.track_sim3(sp, init13=sp.frame_to_ref13, double=True)
    ang, dist, ds = lsdo.sim3_error(lsdg._pose13((Tg, sg)), o)
    assert ang < 1e-4 and dist < 1e-4 and ds < 1e-4, (ang, dist, ds)


def test_sim3_batch_matches_oracle(ctx):
    import lsdg
    sps = [spair(s, 320, 240) for s in range(4)] + [spair(s) for s in range(2)]
    b = lsdg.Batch(ctx, [q.w for q in sps], [q.h for q in sps], [q.intr for q in sps], sim3=True)
    try:
        init = np.tile(np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]]), (len(sps), 1))
        b.load_sim3(*lsdg.pack_sim3_pairs(sps), init)
        b.run()
        out, stats = b.read()
        for i, q in enumerate(sps):
            rc, o, _ = lsdo.track_sim3(q, double=True)
            assert stats[i].status == rc == 0
            ang, dist, ds = lsdo.sim3_error(out[i], o)
            assert ang < 1e-4 and dist < 1e-4 and ds < 1e-4, (i, ang, dist, ds)
        # a second run of the captured graph reproduces the first bit for bit
        b.run()
        out2, _ = b.read()
        np.testing.assert_array_equal(out, out2)
    finally:
        b.close()


def test_sim3_argument_checks(ctx):
    import lsdg
    import lsdg_types as T
    sp = spair(0, 320, 240)
    ref, cur = frames(ctx, sp)
    bad = np.concatenate([np.eye(3).ravel(), np.zeros(3), [0.0]])
    with pytest.raises(lsdg.LsdgError) as e:
        lsdg.sim3_normal_equations(ctx, ref, cur, 0, bad)
    assert e.value.status == T.INVALID_ARG
    nodepth = lsdg.Frame(ctx, sp.w, sp.h, sp.intr).upload(sp.new_image)
    with pytest.raises(lsdg.LsdgError) as e:
        lsdg.Sim3Tracker(ctx).trackFrameSim3(ref, nodepth)
    assert e.value.status == T.INVALID_ARG
    # an SE3 batch refuses Sim3 loads and the other way round
    b = lsdg.Batch(ctx, [sp.w], [sp.h], [sp.intr])
    with pytest.raises(lsdg.LsdgError):
        b.load_sim3(*lsdg.pack_sim3_pairs([sp]), np.zeros((1, 13)))
    b.close()


def test_sim3_batch_from_resident_frames_equals_host_load(ctx):
    """lsdg_batch_load_frames (device-to-device from resident keyframes) gives the results of the
    host upload bit for bit."""
    import lsdg
    sps = [spair(s, 320, 240) for s in range(3)]
    init = np.tile(np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]]), (3, 1))
    b = lsdg.Batch(ctx, [320] * 3, [240] * 3, [q.intr for q in sps], sim3=True)
    try:
        b.load_sim3(*lsdg.pack_sim3_pairs(sps), init)
        b.run()
        ref, _ = b.read()
        pairs = [frames(ctx, q) for q in sps]
        b.load_frames([p[0] for p in pairs], [p[1] for p in pairs], init)
        b.run()
        got, stats = b.read()
        np.testing.assert_array_equal(got, ref)
        with pytest.raises(lsdg.LsdgError):
            b.load_frames([pairs[0][0]] * 3, [lsdg.Frame(ctx, 320, 240, sps[0].intr).upload(sps[0].new_image)] * 3,
                          init)   # Sim3 frames need depth
    finally:
        b.close()
