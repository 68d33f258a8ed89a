"""CPU tests of the tracking oracle: pinned against an independent numpy restatement (bit for bit),
float vs FP64 agreement, and convergence to the synthetic ground truth."""
import numpy as np
import pytest

import lsdo
import np_restate
import synth


def test_pyramid_matches_numpy_restatement(pair0):
    ref = np_restate.pyramid(pair0.ref_image, 5)
    got = lsdo.pyramid(pair0.ref_image, 5)
    for l in range(5):
        assert got[l].shape == ref[l].shape
        np.testing.assert_array_equal(got[l], ref[l])


def test_pyramid_double_close_to_float(small_pair):
    f = lsdo.pyramid(small_pair.ref_image, 4)
    d = lsdo.pyramid(small_pair.ref_image, 4, double=True)
    for l in range(4):
        np.testing.assert_allclose(f[l], d[l], rtol=0, atol=1e-3)


def test_keyframe_points_match_numpy_restatement(pair0):
    D, V, P, PV = lsdo.keyframe(pair0.ref_image, pair0.ref_idepth, pair0.ref_idepth_var, pair0.intr, 5)
    Dn, Vn = np_restate.depth_pyramid(pair0.ref_idepth, pair0.ref_idepth_var, 5)
    pyr = np_restate.pyramid(pair0.ref_image, 5)
    pts = np_restate.points(pyr, Dn, Vn, pair0.intr.as_tuple(), 5)
    for l in range(5):
        np.testing.assert_array_equal(D[l], Dn[l])
        np.testing.assert_array_equal(V[l], Vn[l])
        np.testing.assert_array_equal(P[l], pts[l][0])
        np.testing.assert_array_equal(PV[l], pts[l][1])
    # about 60k semi-dense points at level 0, as the workload specifies
    assert 40000 < len(P[0]) < 90000


def test_normal_equations_float_vs_double(pair0):
    T = synth.pose_inv(pair0.frame_to_ref)
    for level in (0, 2, 4):
        f = lsdo.se3_normal_equations(pair0, T, level)
        d = lsdo.se3_normal_equations(pair0, T, level, double=True)
        assert f[28] == pytest.approx(d[28], abs=3)  # points used can differ only at the image border
        scale = np.abs(d[:27]).max()
        np.testing.assert_allclose(f[:27], d[:27], rtol=0, atol=2e-4 * scale)


def test_normal_equations_descent_direction(pair0):
    """The Gauss-Newton step from calculateWarpUpdate lowers the energy (away from the optimum)."""
    import ctypes
    T0 = np.eye(3, 4)
    ne = lsdo.se3_normal_equations(pair0, T0, 3, double=True)
    H = np.zeros((6, 6))
    q = 0
    for i in range(6):
        for j in range(i, 6):
            H[i, j] = H[j, i] = ne[q]
            q += 1
    g = ne[21:27]
    dx = -np.linalg.solve(H, g)
    assert g @ dx < 0
    lib = lsdo.lib()
    T = np.zeros(12)
    lib_exp = lambda xi: _se3_exp(xi)
    T1 = synth.pose_mul(lib_exp(dx), T0)
    ne1 = lsdo.se3_normal_equations(pair0, T1, 3, double=True)
    assert ne1[27] / ne1[28] < ne[27] / ne[28]


@pytest.mark.parametrize("level", [0, 2, 4])
def test_gradient_is_exact_derivative_of_level_energy(pair0, level):
    """2 J^T W r equals the central finite difference of the energy one LM level minimises (variances
    and participating points fixed by the level's first pass).  This consistency is what lets the
    float oracle, the FP64 oracle and the GPU take the same accept/reject decisions."""
    rng = np.random.default_rng(level)
    T0 = synth.pose_mul(synth.random_motion(rng, (0.1, 0.3), (0.002, 0.005)), synth.pose_inv(pair0.frame_to_ref))
    S = lsdo.se3_fixed_energy(pair0, T0, T0, level)
    h = 1e-6
    fd = np.zeros(6)
    for k in range(6):
        e = np.zeros(6)
        e[k] = h
        Ep = lsdo.se3_fixed_energy(pair0, T0, synth.pose_mul(_se3_exp(e), T0), level)
        Em = lsdo.se3_fixed_energy(pair0, T0, synth.pose_mul(_se3_exp(-e), T0), level)
        assert Ep[28] == Em[28] == S[28]
        fd[k] = (Ep[27] - Em[27]) / (2 * h)
    np.testing.assert_allclose(2 * S[21:27], fd, rtol=0, atol=2e-3 * np.abs(fd).max())


def _se3_exp(xi):
    v, w = xi[:3], xi[3:]
    R = synth.rodrigues(w)
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-8:
        V = np.eye(3) + 0.5 * K
    else:
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * K + (th - np.sin(th)) / th ** 3 * (K @ K)
    return synth.pose(R, V @ v)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_track_converges_to_ground_truth(pairs4, seed):
    p = pairs4[seed]
    rc, T, st = lsdo.track_se3(p)
    assert rc == 0, st.as_dict()
    ang, dist = synth.pose_error(T, p.frame_to_ref)
    # limited by the 5 % inverse-depth noise and sigma=2 image noise of the synthetic keyframe
    assert ang < 3e-3 and dist < 1.5e-2, (ang, dist)
    assert st.good_ratio > 0.8 and st.usage > 0.8
    rcd, Td, std = lsdo.track_se3(p, double=True)
    a2, d2 = synth.pose_error(T, Td)
    assert a2 < 1e-5 and d2 < 1e-5
    assert st.total_passes <= sum(n + 1 for n in lsdo.default_params().max_iterations[:5])


def test_track_identity_pair_stays_at_identity(pair0):
    import copy
    p = copy.copy(pair0)
    p.new_image = pair0.ref_image.copy()
    rc, T, st = lsdo.track_se3(p)
    ang, dist = synth.pose_error(T, np.eye(3, 4))
    assert ang < 1e-4 and dist < 1e-4


def test_track_without_depth_is_lost(small_pair):
    import copy
    p = copy.copy(small_pair)
    p.ref_idepth = np.full_like(small_pair.ref_idepth, -1.0)
    rc, T, st = lsdo.track_se3(p)
    assert rc == 2  # TRACKING_LOST
    assert st.total_passes == 0
    np.testing.assert_allclose(T, np.eye(3, 4))


def test_multithreaded_pass_matches_single_thread(pair0):
    rc1, T1, _ = lsdo.track_se3(pair0, threads=1)
    rc4, T4, _ = lsdo.track_se3(pair0, threads=4)
    a, d = synth.pose_error(T1, T4)
    assert a < 1e-5 and d < 1e-5


def test_cpu_batch_matches_single_pairs(small_pair):
    pairs = [small_pair, synth.tracking_pair(11, 320, 240)]
    out, stats = lsdo.track_batch(pairs, threads=2)
    for i, p in enumerate(pairs):
        rc, T, st = lsdo.track_se3(p)
        np.testing.assert_array_equal(out[i], T)
        assert stats[i].total_passes == st.total_passes
