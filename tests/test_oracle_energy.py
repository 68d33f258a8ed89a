"""CPU tests of the photometric-energy oracle: the FP64 adjoint against FP64 central finite
differences (h = 1e-4 on the twist, 1e-5 on inverse depth, 1,000 random inverse-depth coordinates),
the pose gradient against the calculateWarpUpdate record (dE/dxi = 2 sum w J^T r), float vs FP64,
and the inverse-depth refinement (energy decreases, float close to FP64)."""
import numpy as np
import pytest

import lsdo
import synth

H_TWIST = 1e-4
H_IDEPTH = 1e-5


@pytest.fixture(scope="module")
def epair():
    return synth.tracking_pair(0)


@pytest.fixture(scope="module")
def rprob():
    return synth.refine_problem(0)


def _E(p, T, **kw):
    return lsdo.energy(p.ref_image, p.ref_idepth, p.ref_idepth_var, p.new_image, p.intr, p.w, p.h, T, **kw)


def _left(xi, T):
    """exp(xi) * T for a 6- or 7-vector twist (sim3_exp with sigma = 0 is the SE3 exp)."""
    x = np.zeros(7)
    x[:len(xi)] = xi
    A = np.vstack([lsdo.sim3_exp(x), [0, 0, 0, 1]])
    B = np.vstack([np.asarray(T).reshape(3, 4), [0, 0, 0, 1]])
    return (A @ B)[:3]


def twist_fd(p, T, act, dof, h):
    fd = np.zeros(dof)
    for k in range(dof):
        e = np.zeros(dof)
        e[k] = h
        Ep = _E(p, _left(e, T), dof=dof, fixed_active=act, grad=False, double=True)
        Em = _E(p, _left(-e, T), dof=dof, fixed_active=act, grad=False, double=True)
        assert Ep["broken"] == 0 and Em["broken"] == 0
        fd[k] = (Ep["E"] - Em["E"]) / (2 * h)
    return fd


@pytest.mark.parametrize("dof", [6, 7])
def test_twist_gradient_matches_central_differences(epair, dof):
    """The energy is C1 but not C2: the Catmull-Rom interpolant's second derivative jumps at pixel
    borders and the Huber norm's at its threshold.  A central difference therefore carries an O(h)
    error from the points whose h-neighbourhood straddles such a kink (about 2e-3 of the gradient
    at h = 1e-4), and converges to the adjoint as h shrinks (checked at 1e-6)."""
    T = synth.pose_inv(epair.frame_to_ref)
    base = _E(epair, T, dof=dof, double=True)
    act = base["active"]
    g = base["gxi"]
    fd = twist_fd(epair, T, act, dof, H_TWIST)
    np.testing.assert_allclose(g, fd, rtol=0, atol=5e-3 * np.abs(fd).max())
    fd6 = twist_fd(epair, T, act, dof, 1e-6)
    np.testing.assert_allclose(g, fd6, rtol=0, atol=5e-5 * np.abs(fd).max())


def test_idepth_gradient_matches_central_differences(epair):
    T = synth.pose_inv(epair.frame_to_ref)
    base = _E(epair, T, double=True)
    act = base["active"]
    pix, rho0 = lsdo.energy_points(epair.ref_image, epair.ref_idepth, epair.ref_idepth_var, epair.intr, epair.w,
                                   epair.h)
    rng = np.random.default_rng(0)
    pts = rng.choice(np.nonzero(act)[0], 1000, replace=False)
    # the energy is a sum of per-point terms: shifting every rho by +-h moves each term by its own
    # derivative, so one pair of evaluations gives all the per-point differences at once
    rp = (rho0.astype(np.float64) + H_IDEPTH).astype(np.float32)
    rm = (rho0.astype(np.float64) - H_IDEPTH).astype(np.float32)
    Ep = _E(epair, T, rho=rp, fixed_active=act, grad=False, double=True)
    Em = _E(epair, T, rho=rm, fixed_active=act, grad=False, double=True)
    h_eff = (rp.astype(np.float64) - rm.astype(np.float64)) / 2  # the float32 steps actually taken
    fd = (Ep["e_point"] - Em["e_point"]) / (2 * h_eff)
    g = base["grho"]
    scale = np.abs(g[act > 0]).max()
    err = np.abs(g[pts] - fd[pts])
    assert err.max() < 1e-3 * scale, (err.max(), scale)
    assert np.median(err / np.maximum(np.abs(fd[pts]), 1e-3 * scale)) < 1e-4


def test_pose_gradient_is_twice_the_warp_update(epair):
    """With the tracker's residual variance equal to the photometric variance (keyframe variance
    negligible), dE/dxi = 2 sum w J^T r of calculateWarpUpdate, same points, same weights."""
    import dataclasses
    p = dataclasses.replace(epair, ref_idepth_var=np.where(epair.ref_idepth_var > 0, np.float32(1e-30),
                                                           np.float32(-1)).astype(np.float32))
    T = synth.pose_inv(epair.frame_to_ref)
    # level 0: the same inverse depths, equal up to FP64 rounding (the two codes associate w J r
    # differently and the sums cancel); level 2: the energy's inverse depths are float by contract
    # while the FP64 tracker keeps the averaged depth pyramid in double
    for level, tol in ((0, 1e-6), (2, 1e-5)):
        ne = lsdo.se3_normal_equations(p, T, level, double=True)
        e = _E(p, T, level=level, double=True)
        assert e["n_active"] == int(ne[28])
        np.testing.assert_allclose(e["gxi"], 2 * ne[21:27], rtol=0, atol=tol * np.abs(ne[21:27]).max())
        assert e["E"] == pytest.approx(ne[27], rel=tol * 1e-2)


def test_energy_float_vs_double(epair):
    T = synth.pose_inv(epair.frame_to_ref)
    f = _E(epair, T)
    d = _E(epair, T, double=True)
    assert abs(f["n_active"] - d["n_active"]) <= 2
    assert f["E"] == pytest.approx(d["E"], rel=1e-4)
    np.testing.assert_allclose(f["gxi"], d["gxi"], rtol=0, atol=1e-3 * np.abs(d["gxi"]).max())


def test_refine_lowers_energy_and_matches_fp64(rprob):
    rp = rprob
    args = (rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.frame_images, rp.ref_to_frame, rp.intr, rp.w, rp.h)
    rf, e0f, e1f, nf_ = lsdo.energy_refine(*args)
    rd, e0d, e1d, nd = lsdo.energy_refine(*args, double=True)
    assert e1f < 0.8 * e0f and e1d < 0.8 * e0d
    assert nf_ == nd
    rel = np.abs(rf / rd - 1)
    assert np.median(rel) < 1e-5 and np.mean(rel < 1e-3) > 0.995, (np.median(rel), np.mean(rel < 1e-3))


def test_refine_moves_towards_truth(rprob):
    """MAP refinement of the 5 %-noisy depths with the 8 frames: the median relative error to the
    true inverse depth drops (the frames' 10 cm arc limits how far)."""
    rp = rprob
    pix, rho0 = lsdo.energy_points(rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.intr, rp.w, rp.h)
    truth = rp.true_idepth.ravel()[pix]
    rho, e0, e1, n = lsdo.energy_refine(rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.frame_images,
                                        rp.ref_to_frame, rp.intr, rp.w, rp.h, double=True)
    before = np.median(np.abs(rho0 / truth - 1))
    after = np.median(np.abs(rho / truth - 1))
    assert after < 0.95 * before, (before, after)


def test_refine_without_steps_or_frames_keeps_depths(rprob):
    rp = rprob
    pix, rho0 = lsdo.energy_points(rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.intr, rp.w, rp.h)
    rho, e0, e1, n = lsdo.energy_refine(rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.frame_images[:1],
                                        rp.ref_to_frame[:1], rp.intr, rp.w, rp.h, steps=0)
    np.testing.assert_array_equal(rho, rho0)
    assert e0 == e1
