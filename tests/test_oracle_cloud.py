"""CPU tests of the point-cloud oracle (Keyframe::computeVbo restated, Keyframe.h:66-143): known
answers worked out by hand from the reference's loop, and an independent vectorised numpy
restatement that must agree bit for bit on random inputs."""
import numpy as np
import pytest

import lsdo
import lsdg_types as T

W, H = 64, 48
K = (60.0, 58.0, 31.5, 23.25)


def dense(idepth, var, color=None):
    h, w = idepth.shape
    p = np.zeros((h, w), lsdo.POINT_DENSE)
    p["idepth"] = idepth
    p["idepth_var"] = var
    if color is None:
        color = np.arange(w * h, dtype=np.uint32).reshape(h, w) % 251
    for k in range(4):
        p["color"][..., k] = (np.asarray(color, np.uint32) + 40 * k) % 256
    return p


def numpy_cloud(points, fx, fy, cx, cy, scale, sth=np.float32(1e-3), ath=np.float32(1e-1), minsup=9):
    """Independent restatement: float32 numpy, whole-image masks, row-major order."""
    f32 = np.float32
    h, w = points.shape
    d = points["idepth"].astype(f32)
    v = points["idepth_var"].astype(f32)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        depth = f32(1) / d
        d4 = depth * depth
        d4 = d4 * d4
        keep = ~(d <= 0)
        keep &= ~(v * d4 > sth)
        keep &= ~(((v * d4) * f32(scale)) * f32(scale) > ath)
        back = f32(1) / depth
        sup = np.zeros((h, w), np.int32)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                nb = np.zeros_like(d)
                nb[max(0, -dy):h - max(0, dy), max(0, -dx):w - max(0, dx)] = \
                    d[max(0, dy):h - max(0, -dy), max(0, dx):w - max(0, -dx)]
                diff = nb - back
                sup += ((nb > 0) & (diff * diff < f32(2) * v)).astype(np.int32)
        if minsup > 1:
            keep &= sup >= minsup
    keep[0, :] = keep[-1, :] = False
    keep[:, 0] = keep[:, -1] = False
    ys, xs = np.nonzero(keep)
    fxi, fyi = f32(1) / f32(fx), f32(1) / f32(fy)
    cxi, cyi = -f32(cx) / f32(fx), -f32(cy) / f32(fy)
    out = np.zeros(len(xs), lsdo.CLOUD_VERTEX)
    dep = depth[ys, xs]
    out["point"][:, 0] = (xs.astype(f32) * fxi + cxi) * dep
    out["point"][:, 1] = (ys.astype(f32) * fyi + cyi) * dep
    out["point"][:, 2] = dep
    c = points["color"][ys, xs]
    out["color"][:, 0] = c[:, 2]
    out["color"][:, 1] = c[:, 1]
    out["color"][:, 2] = c[:, 0]
    out["color"][:, 3] = 100
    return out


def random_keyframe(seed, w=W, h=H):
    """Smooth surfaces with noise, holes and a range of variances, so that every filter branch and
    support counts around the threshold of 9 occur."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    idepth = 0.5 + 0.1 * np.sin(xx / 40.0) * np.cos(yy / 30.0)
    idepth *= 1 + 0.002 * rng.normal(size=(h, w))
    idepth[rng.random((h, w)) < 0.02] = -1.0
    idepth[rng.random((h, w)) < 0.005] = 0.0
    var = 10 ** rng.uniform(-6.5, -4, size=(h, w))
    color = rng.integers(0, 256, size=(h, w))
    return dense(idepth.astype(np.float32), var.astype(np.float32), color)


def test_defaults_are_computevbo_constants():
    p = T.CloudParams()
    # Keyframe.h:78-82: my_scaledTH = 1e-3, my_absTH = 1e-1, my_minNearSupport = 9
    import lsdg
    lsdg.lib().lsdg_cloud_default_params(p)
    assert p.scaled_th == np.float32(1e-3) and p.abs_th == np.float32(1e-1) and p.min_near_support == 9


def test_known_answers():
    # 5x5 keyframe at inverse depth 0.5 everywhere, small variance: only pixels whose whole 3x3
    # neighbourhood is inside the image (and so supports them with 9) survive -> the 3x3 interior.
    idepth = np.full((5, 5), 0.5, np.float32)
    var = np.full((5, 5), 1e-5, np.float32)
    pts = dense(idepth, var, np.full((5, 5), 7))
    fx, fy, cx, cy = 10.0, 20.0, 2.0, 2.0
    v = lsdo.cloud_build(pts, 5, 5, fx, fy, cx, cy)
    assert len(v) == 9
    # row-major order: (1,1), (2,1), (3,1), (1,2) ...
    np.testing.assert_array_equal(v["point"][:, 2], np.float32(2.0))
    x = np.array([1, 2, 3] * 3, np.float32)
    y = np.repeat(np.array([1, 2, 3], np.float32), 3)
    np.testing.assert_array_equal(v["point"][:, 0], (x * np.float32(0.1) + np.float32(-0.2)) * np.float32(2))
    np.testing.assert_array_equal(v["point"][:, 1], (y * np.float32(0.05) + np.float32(-0.1)) * np.float32(2))
    # colour swizzle: [0] = input[2], [1] = input[1], [2] = input[0], [3] = 100
    assert list(v["color"][0]) == [(7 + 80) % 256, 7 + 40, 7, 100]
    # a hole at (x=2, y=1) removes the support of every pixel whose 3x3 neighbourhood contains it
    # (rows y = 1 and 2); row y = 3 keeps its three points
    idepth[1, 2] = -1
    v = lsdo.cloud_build(dense(idepth, var), 5, 5, fx, fy, cx, cy)
    assert len(v) == 3
    np.testing.assert_array_equal(v["point"][:, 1], (np.float32(3) * np.float32(0.05) + np.float32(-0.1)) * np.float32(2))
    # variance threshold: var * depth^4 > 1e-3 drops the point (depth 2 -> factor 16)
    idepth[1, 2] = 0.5
    var2 = var.copy()
    var2[2, 2] = 1e-3 / 16 * 1.01
    v = lsdo.cloud_build(dense(idepth, var2), 5, 5, fx, fy, cx, cy)
    assert len(v) == 8 and not np.any((v["point"][:, 0] == 0) & (v["point"][:, 1] == 0))
    # absolute threshold: var * depth^4 * scale^2 > 1e-1 drops the point
    v = lsdo.cloud_build(dense(idepth, var), 5, 5, fx, fy, cx, cy, scale=20.0)
    assert len(v) == 9  # 1e-5 * 16 * 400 = 0.064
    v = lsdo.cloud_build(dense(idepth, var), 5, 5, fx, fy, cx, cy, scale=30.0)
    assert len(v) == 0  # 1e-5 * 16 * 900 = 0.144
    # support 1 keeps every interior point with depth
    v = lsdo.cloud_build(dense(idepth, var), 5, 5, fx, fy, cx, cy, min_near_support=1)
    assert len(v) == 9


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("scale", [1.0, 12.0])
def test_matches_numpy_restatement(seed, scale):
    pts = random_keyframe(seed)
    got = lsdo.cloud_build(pts, W, H, *K, scale=scale)
    ref = numpy_cloud(pts, *K, scale)
    assert len(got) == len(ref) and len(got) > 100
    assert got.tobytes() == ref.tobytes()


def reference_cases():
    """(points, w, h, fx, fy, cx, cy, scale, vertices) of tests/golden/cloud_ref.npz: outputs of the
    reference's own computeVbo loop compiled from Keyframe.h (tests/golden/make_cloud_ref.py)."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cloud_ref.npz"))
    k = 0
    cases = []
    while f"camera{k}" in z:
        w, h, fx, fy, cx, cy, scale = z[f"camera{k}"]
        pts = np.frombuffer(z[f"points{k}"].tobytes(), lsdo.POINT_DENSE).reshape(int(h), int(w))
        v = np.frombuffer(z[f"vertices{k}"].tobytes(), lsdo.CLOUD_VERTEX)
        cases.append((pts, int(w), int(h), float(fx), float(fy), float(cx), float(cy), float(scale), v))
        k += 1
    return cases


def test_oracle_matches_reference_fixture():
    """The oracle against the reference's own loop, through the committed fixture."""
    cases = reference_cases()
    assert len(cases) == 3
    for pts, w, h, fx, fy, cx, cy, scale, v in cases:
        got = lsdo.cloud_build(pts, w, h, fx, fy, cx, cy, scale=scale)
        assert len(got) == len(v) > 500
        assert got.tobytes() == v.tobytes()


def _edge_keyframes():
    rng = np.random.default_rng(11)
    yield "all holes", dense(np.full((8, 9), -1.0, np.float32), np.full((8, 9), 1e-6, np.float32)), 1.0
    yield "3x3", dense(np.full((3, 3), 0.5, np.float32), np.full((3, 3), 1e-6, np.float32)), 1.0
    yield "2 rows", dense(np.full((2, 7), 0.5, np.float32), np.full((2, 7), 1e-6, np.float32)), 1.0
    yield "zeros and negatives", dense(rng.choice([0.0, -0.0, -2.0, 0.5], size=(12, 10)).astype(np.float32),
                                       np.full((12, 10), 1e-6, np.float32)), 1.0
    flat = np.full((16, 16), 0.25, np.float32)
    var = np.full((16, 16), 1e-3 / 256, np.float32)  # var * depth^4 == 1e-3 exactly at depth 4
    yield "scaled threshold boundary", dense(flat, var), 1.0
    yield "absolute threshold boundary", dense(flat, np.full((16, 16), 1e-6, np.float32)), float(np.sqrt(0.1 / 256e-6))


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
@pytest.mark.parametrize("scale", [0.25, 1.0, 12.0])
def test_oracle_matches_reference_code(seed, scale):
    """The oracle against the reference's own loop compiled from Keyframe.h (oracle/_ref), where the
    reference tree or its generated source is present: random keyframes and edge cases."""
    if lsdo.ref_lib() is None:
        pytest.skip("oracle/_ref not built: the reference tree is absent")
    w, h = (64, 48) if seed < 2 else (160, 120)
    pts = random_keyframe(seed + 100, w, h)
    ref = lsdo.ref_compute_vbo(pts, w, h, *K, scale=scale)
    got = lsdo.cloud_build(pts, w, h, *K, scale=scale)
    assert len(got) == len(ref) > 100
    assert got.tobytes() == ref.tobytes()


def test_oracle_matches_reference_code_edges():
    if lsdo.ref_lib() is None:
        pytest.skip("oracle/_ref not built: the reference tree is absent")
    for name, pts, scale in _edge_keyframes():
        h, w = pts.shape
        ref = lsdo.ref_compute_vbo(pts, w, h, *K, scale=scale)
        got = lsdo.cloud_build(pts, w, h, *K, scale=scale)
        assert got.tobytes() == ref.tobytes(), name
