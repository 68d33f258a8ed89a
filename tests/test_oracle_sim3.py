"""CPU tests of the Sim3 tracking oracle (Sim3Tracker::trackFrameSim3 restatement): the Sim3
exponential against a matrix exponential, the reduction to the SE3 normal equations when the depth
residual is switched off, float vs FP64 agreement and recovery of the synthetic similarity."""
import numpy as np
import pytest
from scipy.linalg import expm

import lsdo
import synth


def _hat(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]], np.float64)


def _sim3_expm(xi):
    """exp of the 4x4 generator [[hat(omega) + sigma I, v], [0, 0]] -> [[s R, t], [0, 1]]."""
    v, w, sg = np.asarray(xi[:3]), np.asarray(xi[3:6]), float(xi[6])
    A = np.zeros((4, 4))
    A[:3, :3] = _hat(w) + sg * np.eye(3)
    A[:3, 3] = v
    return expm(A)[:3, :]


@pytest.fixture(scope="module")
def spair():
    return synth.sim3_pair(3, 320, 240)


def _idx7(i, j):
    i, j = min(i, j), max(i, j)
    return i * 7 - i * (i - 1) // 2 + (j - i)


@pytest.mark.parametrize("xi", [
    [0, 0, 0, 0, 0, 0, 0.3],
    [0.1, -0.2, 0.05, 0, 0, 0, 0],
    [0.1, -0.2, 0.05, 0.3, -0.1, 0.2, 0],
    [0.1, -0.2, 0.05, 0.3, -0.1, 0.2, -0.4],
    [1e-3, 2e-3, -1e-3, 1e-4, -2e-4, 3e-4, 5e-4],       # series branch of both coefficients
    [0.5, 0.1, -0.3, 1.2, 0.4, -0.8, 0.7],               # closed forms
    [0.01, 0.02, 0.03, 0.04, 0.0, 0.0, 1e-9],            # theta on the series border, tiny sigma
    [0.01, 0.02, 0.03, 0.0, 0.0, 0.0, 1.5],              # large sigma, no rotation
    [0.01, 0.02, 0.03, 0.01, -0.02, 0.01, -2.5],          # large negative sigma, small rotation
    [0.3, 0.2, 0.1, 0.03, 0.0, 0.04, 1.0],                # theta = 0.05, sigma = 1: both borders
])
def test_sim3_exp_matches_matrix_exponential(xi):
    got = lsdo.sim3_exp(xi)
    ref = _sim3_expm(xi)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * max(1.0, np.abs(ref).max()))


def test_sim3_reduces_to_se3_without_depth_residual(spair):
    """With sim3_depth_weight = 0 and unit scale, the (v, omega) block of the Sim3 normal
    equations is the SE3 record of the same pose, bit for bit in FP64."""
    p = lsdo.default_params()
    p.sim3_depth_weight = 0.0
    T = synth.pose_inv(np.concatenate([np.reshape(spair.frame_to_ref13[:9], (3, 3)),
                                       np.reshape(spair.frame_to_ref13[9:12], (3, 1))], 1))
    T13 = np.concatenate([T[:, :3].ravel(), T[:, 3], [1.0]])
    for level in (1, 3):
        s7 = lsdo.sim3_normal_equations(spair, T13, level, params=p, double=True)
        s6 = lsdo.se3_normal_equations(spair, T, level, params=p, double=True)
        q = 0
        for i in range(6):
            for j in range(i, 6):
                assert s7[_idx7(i, j)] == s6[q], (i, j)
                q += 1
        np.testing.assert_array_equal(s7[28:34], s6[21:27])
        assert s7[35] == s6[27]
        assert s7[36] == s6[28]


def test_sim3_normal_equations_float_vs_double(spair):
    """Photometric part: float and FP64 agree to single precision.  With the inverse-depth term on,
    the few points whose projection lies within rounding of a pixel border can take different
    bilinear cells in float and FP64; the bilinear derivative of the depth map jumps there and the
    four-corner validity can change, and each such point carries a weight up to
    1/sim3_depth_variance.  The sums then agree only to about 1e-3 of their scale."""
    T13 = np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]])
    p0 = lsdo.default_params()
    p0.sim3_depth_weight = 0.0
    for level in (0, 2):
        f = lsdo.sim3_normal_equations(spair, T13, level, params=p0)
        d = lsdo.sim3_normal_equations(spair, T13, level, params=p0, double=True)
        assert f[36] == pytest.approx(d[36], abs=3)
        scale = np.abs(d[:36]).max()
        np.testing.assert_allclose(f[:36], d[:36], rtol=0, atol=5e-5 * scale)
        f = lsdo.sim3_normal_equations(spair, T13, level)
        d = lsdo.sim3_normal_equations(spair, T13, level, double=True)
        scale = np.abs(d[:36]).max()
        np.testing.assert_allclose(f[:36], d[:36], rtol=0, atol=1e-2 * scale)


@pytest.mark.parametrize("seed", [0, 3])
def test_track_sim3_recovers_similarity(seed):
    sp = synth.sim3_pair(seed, 320, 240)
    rc, out, st = lsdo.track_sim3(sp, double=True)
    assert rc == 0
    ang, dist, ds = lsdo.sim3_error(out, sp.frame_to_ref13)
    # the synthetic maps carry 5 % multiplicative depth noise: the pose is recovered to the
    # accuracy that noise allows, the scale to within 1 %
    assert ang < 5e-3 and dist < 2e-2 and ds < 1e-2, (ang, dist, ds)


def test_track_sim3_float_vs_double(spair):
    rcf, f, _ = lsdo.track_sim3(spair)
    rcd, d, _ = lsdo.track_sim3(spair, double=True)
    assert rcf == rcd == 0
    ang, dist, ds = lsdo.sim3_error(f, d)
    assert ang < 1e-5 and dist < 1e-5 and ds < 1e-5, (ang, dist, ds)


def test_track_sim3_depth_term_pins_scale(spair):
    """The photometric residual alone leaves the scale nearly free; the inverse-depth residual is
    what pins it (the point of Sim3 tracking between keyframes)."""
    p = lsdo.default_params()
    rc, out, st = lsdo.track_sim3(spair, params=p, double=True)
    assert rc == 0
    H = np.zeros((7, 7))
    for i in range(7):
        for j in range(i, 7):
            H[i, j] = H[j, i] = st.hessian[_idx7(i, j)]
    assert H[6, 6] > 0
    p0 = lsdo.default_params()
    p0.sim3_depth_weight = 0.0
    d = lsdo.sim3_normal_equations(spair, out, 0, params=p0, double=True)
    # curvature along log-scale with and without the depth term: the depth term dominates
    assert H[6, 6] > 5 * d[_idx7(6, 6)]
