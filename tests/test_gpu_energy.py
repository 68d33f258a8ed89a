"""GPU parity of the photometric energy (forward / adjoint) and of the inverse-depth refinement,
through the C-ABI: per-point values bit-identical to the float oracle (both without FMA
contraction), the pose gradient against the FP64 oracle, central finite differences and the
calculateWarpUpdate record, the autograd-Function contract, and the refinement against the float
and FP64 oracles."""
import numpy as np
import pytest

import lsdo
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def epair():
    return synth.tracking_pair(0)


@pytest.fixture(scope="module")
def rprob():
    return synth.refine_problem(0)


def frames(ctx, p):
    import lsdg
    kf = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.ref_image).set_depth(p.ref_idepth, p.ref_idepth_var)
    f = lsdg.Frame(ctx, p.w, p.h, p.intr).upload(p.new_image)
    return kf, f


def _E(p, T, **kw):
    return lsdo.energy(p.ref_image, p.ref_idepth, p.ref_idepth_var, p.new_image, p.intr, p.w, p.h, T, **kw)


@pytest.mark.parametrize("level", [0, 1, 3])
def test_forward_backward_match_float_oracle(ctx, epair, level):
    import lsdg
    kf, f = frames(ctx, epair)
    T = synth.pose_inv(epair.frame_to_ref)
    en = lsdg.PhotometricEnergy(ctx, kf, level)
    try:
        o = _E(epair, T, level=level)
        pix, rho0 = lsdo.energy_points(epair.ref_image, epair.ref_idepth, epair.ref_idepth_var, epair.intr, epair.w,
                                       epair.h, level)
        assert en.n == len(pix)
        np.testing.assert_array_equal(en.pixels(), pix)
        np.testing.assert_array_equal(en.idepth(), rho0)
        E = en.forward(f, T)
        assert en.n_active == o["n_active"]
        assert E == pytest.approx(o["E"], rel=1e-6)
        gxi, grho = en.backward(1.0)
        # per-point adjoint: the same float operations as the oracle, bit for bit
        np.testing.assert_array_equal(grho, o["grho"].astype(np.float32))
        np.testing.assert_allclose(gxi, o["gxi"], rtol=0, atol=1e-5 * np.abs(o["gxi"]).max())
    finally:
        en.close()


def test_adjoint_against_fp64_finite_differences(ctx, epair):
    """GPU adjoint (float) against FP64 central differences: h = 1e-4 on the twist (the O(h) kink
    error of the C1 energy is ~2e-3 of the gradient there), h = 1e-5 on 1,000 random inverse depths."""
    import lsdg
    from test_oracle_energy import twist_fd
    kf, f = frames(ctx, epair)
    T = synth.pose_inv(epair.frame_to_ref)
    en = lsdg.PhotometricEnergy(ctx, kf, 0)
    try:
        en.forward(f, T)
        gxi, grho = en.backward(1.0)
    finally:
        en.close()
    base = _E(epair, T, double=True)
    act = base["active"]
    fd = twist_fd(epair, T, act, 6, 1e-4)
    np.testing.assert_allclose(gxi, fd, rtol=0, atol=5e-3 * np.abs(fd).max())
    np.testing.assert_allclose(gxi, base["gxi"], rtol=0, atol=2e-4 * np.abs(base["gxi"]).max())
    pix, rho0 = lsdo.energy_points(epair.ref_image, epair.ref_idepth, epair.ref_idepth_var, epair.intr, epair.w,
                                   epair.h)
    rp = (rho0.astype(np.float64) + 1e-5).astype(np.float32)
    rm = (rho0.astype(np.float64) - 1e-5).astype(np.float32)
    Ep = _E(epair, T, rho=rp, fixed_active=act, grad=False, double=True)
    Em = _E(epair, T, rho=rm, fixed_active=act, grad=False, double=True)
    fdr = (Ep["e_point"] - Em["e_point"]) / (rp.astype(np.float64) - rm.astype(np.float64))
    pts = np.random.default_rng(1).choice(np.nonzero(act)[0], 1000, replace=False)
    scale = np.abs(grho).max()
    err = np.abs(grho[pts] - fdr[pts])
    assert err.max() < 1e-3 * scale, (err.max(), scale)


def test_pose_gradient_is_twice_the_gpu_warp_update(ctx, epair):
    """dE/dxi of the energy kernel = 2 x the J^T W r of the tracker's normal-equation kernel when
    the residual variance is the photometric variance (keyframe variance negligible)."""
    import lsdg
    var = np.where(epair.ref_idepth_var > 0, np.float32(1e-30), np.float32(-1)).astype(np.float32)
    kf = lsdg.Frame(ctx, epair.w, epair.h, epair.intr).upload(epair.ref_image).set_depth(epair.ref_idepth, var)
    f = lsdg.Frame(ctx, epair.w, epair.h, epair.intr).upload(epair.new_image)
    T = synth.pose_inv(epair.frame_to_ref)
    ne = lsdg.se3_normal_equations(ctx, kf, f, 0, T)
    en = lsdg.PhotometricEnergy(ctx, kf, 0)
    try:
        E = en.forward(f, T)
        gxi, _ = en.backward(1.0, want_idepth=False)
    finally:
        en.close()
    assert en.n_active == int(ne[28])
    # the tracker is compiled with FMA contraction, the energy kernel without: float-level agreement
    np.testing.assert_allclose(gxi, 2 * ne[21:27], rtol=0, atol=5e-5 * np.abs(ne[21:27]).max())
    assert E == pytest.approx(ne[27], rel=1e-5)


def test_sim3_dof_gradient(ctx, epair):
    import lsdg
    kf, f = frames(ctx, epair)
    T = synth.pose_inv(epair.frame_to_ref)
    en = lsdg.PhotometricEnergy(ctx, kf, 0)
    try:
        en.forward(f, T, dof=7)
        gxi, grho = en.backward(1.0)
    finally:
        en.close()
    o = _E(epair, T, dof=7)
    assert gxi.shape == (7,)
    np.testing.assert_allclose(gxi, o["gxi"], rtol=0, atol=1e-5 * np.abs(o["gxi"]).max())


def test_autograd_contract(ctx, epair):
    import lsdg
    import lsdg_types as Ty
    kf, f = frames(ctx, epair)
    T = synth.pose_inv(epair.frame_to_ref)
    en = lsdg.PhotometricEnergy(ctx, kf, 1)
    try:
        with pytest.raises(lsdg.LsdgError) as e:
            en.backward(1.0)
        assert e.value.status == Ty.INVALID_ARG
        en.forward(f, T)
        g1, r1 = en.backward(1.0)
        g2, r2 = en.backward(-2.5)   # the backward is linear in dL/dE and repeatable
        np.testing.assert_allclose(g2, -2.5 * g1, rtol=1e-6)
        np.testing.assert_array_equal(r2, (np.float32(-2.5) * r1).astype(np.float32))
        rho = en.idepth()
        en.set_idepth(rho * 1.01)    # a saved input changed after the forward
        with pytest.raises(lsdg.LsdgError) as e:
            en.backward(1.0)
        assert e.value.status == Ty.INVALID_ARG
        E1 = en.forward(f, T)
        en.set_idepth(None)
        E0 = en.forward(f, T)
        assert E1 != E0
        # a per-point variance of 4x the photometric variance: inlier terms scale by 1/4
        en.set_sigma2(np.full(en.n, 4 * ctx.params.photometric_variance, np.float32))
        E4 = en.forward(f, T)
        assert E4 < E0
        with pytest.raises(lsdg.LsdgError):
            en.set_sigma2(np.zeros(en.n, np.float32))
        with pytest.raises(lsdg.LsdgError):
            en.forward(f, T, dof=5)
    finally:
        en.close()


def test_refine_matches_oracles(ctx, rprob):
    import lsdg
    rp = rprob
    kf = lsdg.Frame(ctx, rp.w, rp.h, rp.intr).upload(rp.key_image).set_depth(rp.key_idepth, rp.key_idepth_var)
    fs = [lsdg.Frame(ctx, rp.w, rp.h, rp.intr).upload(im) for im in rp.frame_images]
    en = lsdg.PhotometricEnergy(ctx, kf, 0)
    try:
        e0, e1, nref = en.refine(fs, rp.ref_to_frame, 50)
        rho = en.idepth()
    finally:
        en.close()
    args = (rp.key_image, rp.key_idepth, rp.key_idepth_var, rp.frame_images, rp.ref_to_frame, rp.intr, rp.w, rp.h)
    rf, e0f, e1f, nf_ = lsdo.energy_refine(*args)
    rd, e0d, e1d, nd = lsdo.energy_refine(*args, double=True)
    assert nref == nf_
    # the per-point Newton iterations are the same float operations: bit-identical inverse depths
    mism = np.nonzero(rho != rf)[0]
    assert len(mism) == 0, (len(mism), rho[mism[:5]], rf[mism[:5]])
    assert e0 == pytest.approx(e0f, rel=1e-6) and e1 == pytest.approx(e1f, rel=1e-6)
    # against the FP64 oracle: inverse depth within 1e-3 relative for >= 99.5 % of the points
    rel = np.abs(rho / rd - 1)
    assert np.mean(rel < 1e-3) >= 0.995 and np.median(rel) < 1e-5, (np.mean(rel < 1e-3), np.median(rel))
    assert e1 < 0.8 * e0
