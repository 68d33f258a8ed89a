"""Seeded synthetic scenes for the LSD-SLAM hot path (tracking pairs and depth-filter sequences).

The reference ships no dataset (the LSD_room and NOAA sequences its Rakefile and sample config
point at are not distributed with it), so every workload is rendered here from a seed:

* a scene of textured planar patches at 1-5 m in front of the keyframe camera, textured with
  4-octave value noise mapped to [0, 255] (own lattice hash, own smoothstep interpolation);
* pinhole cameras (fx = fy = 500, cx = 320, cy = 240 at 640x480, scaled with the image size);
* a second view after a 1-3 deg rotation about a random axis plus a 2-5 cm translation;
* sigma = 2 Gaussian pixel noise on every rendered image;
* a semi-dense keyframe inverse depth on pixels whose central-difference gradient magnitude
  exceeds 5, perturbed by 5 % relative Gaussian noise, with variance 0.01.

Conventions (the ones the reference's viewer uses, lib/Pangolin_IOWrapper/Keyframe.h:86-89,134-136):
pixel (x, y) back-projects to ((x - cx) / fx * z, (y - cy) / fy * z, z) with z = 1 / idepth, pixel
centres at integer coordinates, images row-major float32 ``[h, w]``.

Poses are 3x4 row-major ``[R | t]`` (float64).  ``frame_to_ref`` maps a point from the second
(tracked) camera into the keyframe camera; it is the quantity ``SE3Tracker::trackFrame`` returns.

This module is data generation for tests and benchmarks; it never runs on the hot path.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

BASE_W, BASE_H = 640, 480
BASE_F, BASE_CX, BASE_CY = 500.0, 320.0, 240.0


@dataclasses.dataclass
class Intrinsics:
    fx: float
    fy: float
    cx: float
    cy: float

    @staticmethod
    def for_size(w: int, h: int) -> "Intrinsics":
        """Intrinsics of the 640x480 reference camera scaled to a w x h image.

        Scaling keeps pixel centres consistent: a w/640 zoom maps continuous coordinate
        x + 0.5 to s * (x + 0.5), so cx' = s * (cx + 0.5) - 0.5.
        """
        sx, sy = w / BASE_W, h / BASE_H
        return Intrinsics(BASE_F * sx, BASE_F * sy, sx * (BASE_CX + 0.5) - 0.5, sy * (BASE_CY + 0.5) - 0.5)

    def as_tuple(self):
        return (self.fx, self.fy, self.cx, self.cy)


# ----------------------------------------------------------------------------------------------
# Small SE3 helpers (float64, numpy)
# ----------------------------------------------------------------------------------------------

def rodrigues(axis_angle: np.ndarray) -> np.ndarray:
    w = np.asarray(axis_angle, dtype=np.float64)
    th = float(np.linalg.norm(w))
    if th < 1e-12:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * (K @ K)


def pose(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    T = np.zeros((3, 4))
    T[:, :3] = R
    T[:, 3] = t
    return T


def pose_inv(T: np.ndarray) -> np.ndarray:
    R = T[:, :3]
    t = T[:, 3]
    return pose(R.T, -R.T @ t)


def pose_mul(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    return pose(A[:, :3] @ B[:, :3], A[:, :3] @ B[:, 3] + A[:, 3])


def pose_error(A: np.ndarray, B: np.ndarray):
    """(rotation angle [rad], translation distance [m]) between two 3x4 poses.  The angle is
    atan2(|vee(dR - dR^T)| / 2, (tr dR - 1) / 2), accurate for small angles too."""
    dR = A[:, :3].T @ B[:, :3]
    c = (np.trace(dR) - 1.0) * 0.5
    v = np.array([dR[2, 1] - dR[1, 2], dR[0, 2] - dR[2, 0], dR[1, 0] - dR[0, 1]]) * 0.5
    ang = math.atan2(float(np.linalg.norm(v)), float(c))
    return ang, float(np.linalg.norm(A[:, 3] - B[:, 3]))


# ----------------------------------------------------------------------------------------------
# Value noise
# ----------------------------------------------------------------------------------------------

def _hash01(ix: np.ndarray, iy: np.ndarray, seed: int) -> np.ndarray:
    """Integer lattice hash -> [0, 1).  Own mixing constants (odd multipliers, xor-shifts)."""
    x = ix.astype(np.int64).astype(np.uint32)
    y = iy.astype(np.int64).astype(np.uint32)
    with np.errstate(over="ignore"):
        h = (x * np.uint32(0x9E3779B1)) ^ (y * np.uint32(0x85EBCA77)) ^ np.uint32((seed * 0xC2B2AE3D + 0x27D4EB2F) & 0xFFFFFFFF)
        h ^= h >> np.uint32(15)
        h *= np.uint32(0x2C1B3C6D)
        h ^= h >> np.uint32(12)
        h *= np.uint32(0x297A2D39)
        h ^= h >> np.uint32(15)
    return h.astype(np.float64) * (1.0 / 4294967296.0)


def value_noise(u: np.ndarray, v: np.ndarray, seed: int, octaves: int = 4, base_freq: float = 1.0,
                footprint: np.ndarray = None) -> np.ndarray:
    """Sum of ``octaves`` octaves of lattice value noise, normalised to [0, 1].  ``footprint``
    (optional, per sample, in texture units): octaves with more than 1/4 cycle per footprint fade
    out linearly, gone at 1/2 (band-limited texture, so a point-sampled render does not alias)."""
    total = np.zeros_like(u)
    amp, norm, f = 1.0, 0.0, base_freq
    for o in range(octaves):
        if footprint is not None:
            c = f * footprint
            fade = np.clip(2.0 - 4.0 * c, 0.0, 1.0)
        else:
            fade = 1.0
        x = u * f
        y = v * f
        ix = np.floor(x)
        iy = np.floor(y)
        fx = x - ix
        fy = y - iy
        sx = fx * fx * (3.0 - 2.0 * fx)
        sy = fy * fy * (3.0 - 2.0 * fy)
        s = seed * 131 + o
        h00 = _hash01(ix, iy, s)
        h10 = _hash01(ix + 1, iy, s)
        h01 = _hash01(ix, iy + 1, s)
        h11 = _hash01(ix + 1, iy + 1, s)
        a = h00 + (h10 - h00) * sx
        b = h01 + (h11 - h01) * sx
        total += (amp * fade) * (a + (b - a) * sy) + (amp * (1.0 - fade)) * 0.5
        norm += amp
        amp *= 0.5
        f *= 2.0
    return total / norm


# ----------------------------------------------------------------------------------------------
# Scene of planar patches
# ----------------------------------------------------------------------------------------------

@dataclasses.dataclass
class Patch:
    centre: np.ndarray      # (3,) in keyframe-camera coordinates
    normal: np.ndarray      # (3,) unit, facing the camera (normal . centre < 0)
    e1: np.ndarray          # (3,) in-plane axis
    e2: np.ndarray          # (3,) in-plane axis
    half: tuple             # half extents along e1, e2 (inf for the background plane)
    tex_seed: int
    tex_freq: float         # value-noise base frequency in cycles per metre
    contrast: float
    offset: float


def _tilted_normal(rng: np.random.Generator, max_tilt_deg: float) -> np.ndarray:
    tilt = math.radians(rng.uniform(0.0, max_tilt_deg))
    az = rng.uniform(0.0, 2 * math.pi)
    n = np.array([math.sin(tilt) * math.cos(az), math.sin(tilt) * math.sin(az), -math.cos(tilt)])
    return n / np.linalg.norm(n)


def _basis(n: np.ndarray):
    a = np.array([1.0, 0.0, 0.0]) if abs(n[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    e1 = np.cross(n, a)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(n, e1)
    return e1, e2


def make_scene(rng: np.random.Generator, n_planes: int = 6, depth_range=(1.0, 5.0), span: float = 1.0):
    """``n_planes`` textured planes at depths in ``depth_range``: one background plane near the
    far end (so every ray hits something) and ``n_planes - 1`` finite patches in front of it.
    ``span`` scales the lateral placement of the patches (the room sequence uses more)."""
    zmin, zmax = depth_range
    patches = []
    n = _tilted_normal(rng, 12.0)
    zb = rng.uniform(zmax - 0.6, zmax)
    c = np.array([0.0, 0.0, zb])
    e1, e2 = _basis(n)
    patches.append(Patch(c, n, e1, e2, (math.inf, math.inf), int(rng.integers(1 << 30)),
                         float(rng.uniform(1.3, 1.7)), float(rng.uniform(0.75, 0.85)), 0.0))
    for _ in range(n_planes - 1):
        z = rng.uniform(zmin, zmax - 0.7)
        # aim at a random point of the 640x480 field of view
        px = rng.uniform(-0.55, 0.55) * span
        py = rng.uniform(-0.45, 0.45) * span
        c = np.array([px * z * (BASE_W / 2) / BASE_F * 2, py * z * (BASE_H / 2) / BASE_F * 2, z])
        n = _tilted_normal(rng, 35.0)
        e1, e2 = _basis(n)
        hw = z * rng.uniform(0.15, 0.35) * (BASE_W / BASE_F)
        hh = z * rng.uniform(0.15, 0.35) * (BASE_H / BASE_F)
        patches.append(Patch(c, n, e1, e2, (hw, hh), int(rng.integers(1 << 30)),
                             float(rng.uniform(1.7, 2.3)), float(rng.uniform(0.75, 0.85)), 0.0))
    return patches


def render(patches, intr: Intrinsics, w: int, h: int, cam_to_ref: np.ndarray, antialias: bool = False):
    """Ray-cast the patches.  ``cam_to_ref`` (3x4) is the rendering camera's pose in the scene
    (keyframe) frame.  Returns (image float64 [h,w] before noise, depth z in this camera [h,w]).
    ``antialias``: band-limit the texture to each pixel's footprint on the surface."""
    R = cam_to_ref[:, :3]
    o = cam_to_ref[:, 3]
    xs = (np.arange(w, dtype=np.float64) - intr.cx) / intr.fx
    ys = (np.arange(h, dtype=np.float64) - intr.cy) / intr.fy
    rx, ry = np.meshgrid(xs, ys)
    dirs_cam = np.stack([rx, ry, np.ones_like(rx)], axis=-1)           # z-component 1 => t == depth
    dirs = dirs_cam @ R.T
    best_t = np.full((h, w), np.inf)
    img = np.zeros((h, w))
    for p in patches:
        denom = dirs @ p.normal
        num = float((p.centre - o) @ p.normal)
        with np.errstate(divide="ignore", invalid="ignore"):
            t = num / denom
        hit = (t > 1e-3) & np.isfinite(t) & (t < best_t)
        if not np.any(hit):
            continue
        pts = o + dirs * t[..., None]
        d = pts - p.centre
        a = d @ p.e1
        b = d @ p.e2
        if math.isfinite(p.half[0]):
            hit &= (np.abs(a) <= p.half[0]) & (np.abs(b) <= p.half[1])
        if not np.any(hit):
            continue
        fp = None
        if antialias:
            # footprint of one pixel on the plane: ray length / focal length / |cos incidence|
            dn = np.abs(denom[hit]) / np.linalg.norm(dirs[hit], axis=-1)
            fp = (t[hit] * np.linalg.norm(dirs[hit], axis=-1)) / (intr.fx * np.maximum(dn, 0.05))
        tex = value_noise(a[hit], b[hit], p.tex_seed, 4, p.tex_freq, fp)
        tex = np.clip(0.5 + (tex - 0.5) * 2.2 * p.contrast, 0.0, 1.0) * 255.0
        img[hit] = tex
        best_t[hit] = t[hit]
    depth = best_t  # dirs_cam has unit z, so t is the z-depth in the rendering camera
    return img, depth


def central_gradient(img: np.ndarray):
    """Central-difference gradient, zero on the one-pixel border (the same definition the
    frame pyramid uses)."""
    gx = np.zeros_like(img)
    gy = np.zeros_like(img)
    gx[:, 1:-1] = 0.5 * (img[:, 2:] - img[:, :-2])
    gy[1:-1, :] = 0.5 * (img[2:, :] - img[:-2, :])
    gx[0, :] = 0
    gx[-1, :] = 0
    gy[:, 0] = 0
    gy[:, -1] = 0
    return gx, gy


def random_motion(rng: np.random.Generator, rot_deg=(1.0, 3.0), trans_m=(0.02, 0.05)) -> np.ndarray:
    """frame_to_ref: the second camera's pose in the keyframe camera."""
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = math.radians(rng.uniform(*rot_deg))
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    return pose(rodrigues(axis * ang), d * rng.uniform(*trans_m))


@dataclasses.dataclass
class TrackingPair:
    w: int
    h: int
    intr: Intrinsics
    ref_image: np.ndarray       # float32 [h,w]
    ref_idepth: np.ndarray      # float32 [h,w], <= 0 means no depth
    ref_idepth_var: np.ndarray  # float32 [h,w]
    new_image: np.ndarray       # float32 [h,w]
    frame_to_ref: np.ndarray    # ground truth, float64 3x4
    ref_true_depth: np.ndarray  # float64 [h,w]


def tracking_pair(seed: int = 0, w: int = BASE_W, h: int = BASE_H, noise_sigma: float = 2.0,
                  grad_thresh: float = 5.0, idepth_rel_noise: float = 0.05, idepth_var: float = 0.01,
                  rot_deg=(1.0, 3.0), trans_m=(0.02, 0.05)) -> TrackingPair:
    """One SE3 alignment pair: a keyframe with semi-dense inverse depth and a second view."""
    rng = np.random.default_rng(seed)
    intr = Intrinsics.for_size(w, h)
    patches = make_scene(rng)
    T = random_motion(rng, rot_deg, trans_m)
    img0, depth0 = render(patches, intr, w, h, pose(np.eye(3), np.zeros(3)))
    img1, _ = render(patches, intr, w, h, T)
    img0 = (img0 + rng.normal(0.0, noise_sigma, img0.shape)).astype(np.float32)
    img1 = (img1 + rng.normal(0.0, noise_sigma, img1.shape)).astype(np.float32)
    gx, gy = central_gradient(img0.astype(np.float64))
    sel = (gx * gx + gy * gy) > grad_thresh * grad_thresh
    idepth = np.full((h, w), -1.0)
    noise = 1.0 + idepth_rel_noise * rng.normal(size=(h, w))
    idepth[sel] = (1.0 / depth0[sel]) * noise[sel]
    var = np.where(sel, idepth_var, -1.0)
    return TrackingPair(w, h, intr, img0, idepth.astype(np.float32), var.astype(np.float32), img1, T, depth0)


# The benchmark's workloads, defined once for bench.py and the accuracy tests:
# the headline batch is 64 pairs at 640x480 with seeds 0..63 (rank r of a sharded run: 1000 r + i),
# the mixed batch 20 x 320x240, 32 x 640x480, 12 x 1280x960 with seeds 5000 + i, the Sim3 constraint
# batch 10 pairs at 640x480 with seeds 2000 + i.
HEADLINE_PAIRS = 64
MIXED_SIZES = [(320, 240)] * 20 + [(640, 480)] * 32 + [(1280, 960)] * 12
MIXED_SEED0 = 5000
SIM3_CANDIDATES = 10
SIM3_SEED0 = 2000


def camera_pair(seed: int, w: int = BASE_W, h: int = BASE_H) -> TrackingPair:
    """A tracking pair whose two images are 8-bit values (a camera's format): rounded and clipped
    to 0..255, held as float32."""
    p = tracking_pair(seed, w, h)
    p.ref_image = np.clip(np.rint(p.ref_image), 0, 255).astype(np.float32)
    p.new_image = np.clip(np.rint(p.new_image), 0, 255).astype(np.float32)
    return p


def generate(fn, specs, workers: int):
    """fn(*spec) for every spec in a pool of `workers` spawned processes (never forked: the caller
    may already hold a CUDA context)."""
    import multiprocessing as mp
    if workers <= 1 or len(specs) <= 1:
        return [fn(*s) for s in specs]
    with mp.get_context("spawn").Pool(min(workers, len(specs))) as pool:
        return pool.starmap(fn, specs)


@dataclasses.dataclass
class DepthSequence:
    w: int
    h: int
    intr: Intrinsics
    key_image: np.ndarray          # float32 [h,w]
    key_true_idepth: np.ndarray    # float64 [h,w]
    init_idepth: np.ndarray        # float32 [h,w]
    init_var: np.ndarray           # float32 [h,w]
    ref_images: list               # list of float32 [h,w]
    ref_frame_to_key: list         # list of 3x4 float64: reference camera pose in the keyframe
    next_image: np.ndarray         # float32 [h,w]: the frame that becomes the next keyframe
    next_to_key: np.ndarray        # 3x4


def depth_sequence(seed: int = 0, w: int = BASE_W, h: int = BASE_H, n_refs: int = 8,
                   baseline_m: float = 0.10, noise_sigma: float = 2.0,
                   init_idepth: float = 0.5, init_spread: float = 0.5, init_var: float = 0.5) -> DepthSequence:
    """A keyframe observed by ``n_refs`` reference frames along a smooth arc of ``baseline_m``
    total length (camera centres on a circle segment, gently turning), plus one more frame
    further along the arc that becomes the next keyframe (for propagation)."""
    rng = np.random.default_rng(seed)
    intr = Intrinsics.for_size(w, h)
    patches = make_scene(rng)
    key_img, key_depth = render(patches, intr, w, h, pose(np.eye(3), np.zeros(3)))
    key_img = (key_img + rng.normal(0.0, noise_sigma, key_img.shape)).astype(np.float32)
    # arc in the x-z plane bending slightly, mostly sideways motion with a little forward part
    d = rng.normal(size=3)
    d[2] *= 0.3
    d /= np.linalg.norm(d)
    up = np.cross(d, np.array([0.0, 0.0, 1.0]))
    if np.linalg.norm(up) < 1e-6:
        up = np.array([0.0, 1.0, 0.0])
    up /= np.linalg.norm(up)
    bend = rng.uniform(-0.3, 0.3)
    yaw_total = math.radians(rng.uniform(1.0, 3.0))

    def arc_pose(s):  # s in [0, 1.25]
        c = d * (baseline_m * s) + up * (bend * baseline_m * s * s)
        R = rodrigues(up * (yaw_total * s))
        return pose(R, c)

    refs, poses = [], []
    for k in range(1, n_refs + 1):
        T = arc_pose(k / n_refs)
        im, _ = render(patches, intr, w, h, T)
        refs.append((im + rng.normal(0.0, noise_sigma, im.shape)).astype(np.float32))
        poses.append(T)
    Tn = arc_pose(1.25)
    imn, _ = render(patches, intr, w, h, Tn)
    imn = (imn + rng.normal(0.0, noise_sigma, imn.shape)).astype(np.float32)
    id0 = (init_idepth * (1.0 + rng.uniform(-init_spread, init_spread, (h, w)))).astype(np.float32)
    v0 = np.full((h, w), init_var, dtype=np.float32)
    return DepthSequence(w, h, intr, key_img, 1.0 / key_depth, id0, v0, refs, poses, imn, Tn)


@dataclasses.dataclass
class Sim3Pair:
    """Two keyframes with their own semi-dense inverse depth; keyframe j's map is in its own scale
    (depths multiplied by `scale`), so the true j-to-i transform is a similarity."""
    w: int
    h: int
    intr: Intrinsics
    ref_image: np.ndarray
    ref_idepth: np.ndarray
    ref_idepth_var: np.ndarray
    new_image: np.ndarray
    new_idepth: np.ndarray
    new_idepth_var: np.ndarray
    frame_to_ref13: np.ndarray   # 13 doubles: R (9), t (3), s -- x_i = s R x_j + t


def _semi_dense(rng, img, depth, scale, grad_thresh, rel_noise, var):
    gx, gy = central_gradient(img.astype(np.float64))
    sel = (gx * gx + gy * gy) > grad_thresh * grad_thresh
    idepth = np.full(img.shape, -1.0)
    idepth[sel] = (1.0 / (depth[sel] * scale)) * (1.0 + rel_noise * rng.normal(size=int(sel.sum())))
    return idepth.astype(np.float32), np.where(sel, var, -1.0).astype(np.float32)


def sim3_pair(seed: int = 0, w: int = BASE_W, h: int = BASE_H, scale: float = 1.3, noise_sigma: float = 2.0,
              rel_noise: float = 0.05, idepth_var: float = 0.01) -> Sim3Pair:
    rng = np.random.default_rng(seed)
    intr = Intrinsics.for_size(w, h)
    patches = make_scene(rng)
    T = random_motion(rng)                        # frame j's camera in keyframe i (metric)
    img0, depth0 = render(patches, intr, w, h, pose(np.eye(3), np.zeros(3)))
    img1, depth1 = render(patches, intr, w, h, T)
    img0 = (img0 + rng.normal(0.0, noise_sigma, img0.shape)).astype(np.float32)
    img1 = (img1 + rng.normal(0.0, noise_sigma, img1.shape)).astype(np.float32)
    id0, v0 = _semi_dense(rng, img0, depth0, 1.0, 5.0, rel_noise, idepth_var)
    id1, v1 = _semi_dense(rng, img1, depth1, scale, 5.0, rel_noise, idepth_var / (scale * scale))
    # a point of j's scaled map is x_j' = scale * x_j; x_i = R x_j + t = (1/scale) R x_j' + t
    f2r = np.concatenate([T[:, :3].ravel(), T[:, 3], [1.0 / scale]])
    return Sim3Pair(w, h, intr, img0, id0, v0, img1, id1, v1, f2r)


@dataclasses.dataclass
class RefineProblem:
    """A keyframe with noisy semi-dense inverse depth and frames observing it from known poses."""
    w: int
    h: int
    intr: Intrinsics
    key_image: np.ndarray        # float32 [h,w]
    key_idepth: np.ndarray       # float32 [h,w]: truth x (1 + rel_noise N(0,1)) where |grad| > thresh, else -1
    key_idepth_var: np.ndarray   # float32 [h,w]
    true_idepth: np.ndarray      # float64 [h,w]
    frame_images: list           # float32 [h,w] each
    ref_to_frame: list           # 3x4: keyframe camera -> frame camera


def refine_problem(seed: int = 0, w: int = BASE_W, h: int = BASE_H, n_frames: int = 8, rel_noise: float = 0.05,
                   grad_thresh: float = 5.0) -> RefineProblem:
    """The depth_sequence scene (frames on a smooth 10 cm arc) with the keyframe depth of a tracking
    pair: semi-dense, 5 % multiplicative noise."""
    s = depth_sequence(seed, w, h, n_refs=n_frames)
    rng = np.random.default_rng(seed + 7919)
    gx, gy = central_gradient(s.key_image.astype(np.float64))
    sel = (gx * gx + gy * gy) > grad_thresh * grad_thresh
    idepth = np.full((h, w), -1.0)
    idepth[sel] = s.key_true_idepth[sel] * (1.0 + rel_noise * rng.normal(size=int(sel.sum())))
    # the keyframe's variance is that of its noise (a depth filter's estimate of it)
    var = np.where(sel, (rel_noise * s.key_true_idepth) ** 2, -1.0)
    return RefineProblem(w, h, s.intr, s.key_image, idepth.astype(np.float32), var.astype(np.float32),
                         s.key_true_idepth, list(s.ref_images), [pose_inv(T) for T in s.ref_frame_to_key])


# ----------------------------------------------------------------------------------------------
# A room sequence: 20 textured planes, a closed cubic-spline camera path (full SLAM runs)
# ----------------------------------------------------------------------------------------------

@dataclasses.dataclass
class RoomSequence:
    """Frames of a camera moving through a room; world frame: x right, y down, z forward of the
    room, origin at the room centre (the camera convention, so the first pose is near identity)."""
    w: int
    h: int
    intr: Intrinsics
    fps: float
    patches: list
    cam_to_world: np.ndarray   # (n, 3, 4) ground-truth camera poses
    first_depth: np.ndarray    # float64 [h, w]: z-depth of frame 0 (bootstraps the first keyframe)
    depths: np.ndarray = None  # float32 (n, h, w) z-depth of every frame (keep_depths=True)

    @property
    def n(self) -> int:
        return len(self.cam_to_world)


def make_room(rng: np.random.Generator, size=(8.0, 3.0, 6.0), n_panels: int = 14):
    """6 walls of a box room plus ``n_panels`` vertical panels standing in front of the walls,
    all textured with value noise: 20 planes for the default panel count."""
    sx, sy, sz = size[0] / 2, size[1] / 2, size[2] / 2
    patches = []

    def add(centre, normal, e1, half, freq):
        n = np.asarray(normal, np.float64)
        patches.append(Patch(np.asarray(centre, np.float64), n / np.linalg.norm(n), np.asarray(e1, np.float64),
                             np.cross(n / np.linalg.norm(n), np.asarray(e1, np.float64)), half,
                             int(rng.integers(1 << 30)), freq, float(rng.uniform(0.75, 0.85)), 0.0))

    ex, ey, ez = np.eye(3)
    add([sx, 0, 0], -ex, ez, (sz, sy), float(rng.uniform(3.0, 3.6)))    # walls (normals point inward)
    add([-sx, 0, 0], ex, ez, (sz, sy), float(rng.uniform(3.0, 3.6)))
    add([0, 0, sz], -ez, ex, (sx, sy), float(rng.uniform(3.0, 3.6)))
    add([0, 0, -sz], ez, ex, (sx, sy), float(rng.uniform(3.0, 3.6)))
    add([0, sy, 0], -ey, ex, (sx, sz), float(rng.uniform(3.0, 3.6)))    # floor (y down)
    add([0, -sy, 0], ey, ex, (sx, sz), float(rng.uniform(3.0, 3.6)))    # ceiling
    for _ in range(n_panels):
        ang = rng.uniform(0, 2 * math.pi)
        # a point on an ellipse between the path (radius <= 1.5 m) and the walls, so that every
        # surface stays >= ~1.3 m from the camera (inside the depth filter's default idepth range)
        r = rng.uniform(0.78, 0.92)
        c = np.array([math.cos(ang) * sx * r, rng.uniform(-0.6, 0.6), math.sin(ang) * sz * r])
        yaw = ang + math.pi + rng.uniform(-0.5, 0.5)                      # roughly facing the centre
        n = np.array([math.cos(yaw), 0.0, math.sin(yaw)])
        e1 = np.cross(ey, n)
        add(c, n, e1 / np.linalg.norm(e1), (float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.8))),
            float(rng.uniform(3.6, 4.4)))
    return patches


def room_path(rng: np.random.Generator, n_frames: int, fps: float = 30.0, speed: float = 0.5,
              radius=(1.5, 0.9), look_yaw_deg: float = 35.0):
    """Camera poses along a closed periodic cubic spline through 8 jittered points of an ellipse
    around the room centre, traversed at constant speed; the camera looks outwards, turned
    `look_yaw_deg` towards the direction of travel, with a small pitch."""
    from scipy.interpolate import CubicSpline

    k = 8
    phis = np.arange(k) * 2 * math.pi / k + rng.uniform(-0.15, 0.15, k)
    pts = np.stack([radius[0] * np.cos(phis) * rng.uniform(0.9, 1.1, k), rng.uniform(-0.15, 0.15, k),
                    radius[1] * np.sin(phis) * rng.uniform(0.9, 1.1, k)], 1)
    pts = np.vstack([pts, pts[:1]])
    s = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(pts, axis=0), axis=1))])
    spline = CubicSpline(s, pts, bc_type="periodic")
    # arc-length table for constant speed
    ss = np.linspace(0, s[-1], 20001)
    d = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(spline(ss), axis=0), axis=1))])
    dist = (np.arange(n_frames) * speed / fps) % d[-1]
    u = np.interp(dist, d, ss)
    P = spline(u)
    V = spline(u, 1)
    out = np.zeros((n_frames, 3, 4))
    ey = np.array([0.0, 1.0, 0.0])
    for i in range(n_frames):
        outward = np.array([P[i, 0], 0.0, P[i, 2]])
        outward /= np.linalg.norm(outward)
        vel = np.array([V[i, 0], 0.0, V[i, 2]])
        vel /= np.linalg.norm(vel)
        a = math.radians(look_yaw_deg)
        fwd = math.cos(a) * outward + math.sin(a) * vel
        fwd[1] = 0.08 * math.sin(2 * math.pi * i / 400.0)
        z = fwd / np.linalg.norm(fwd)
        x = np.cross(ey, z)
        x /= np.linalg.norm(x)
        y = np.cross(z, x)
        out[i, :, :3] = np.stack([x, y, z], 1)   # columns: camera axes in the world
        out[i, :, 3] = P[i]
    return out


def _render_u8(args):
    patches, intr, w, h, T, seed, noise_sigma = args
    img, depth = render(patches, intr, w, h, T, antialias=True)
    rng = np.random.default_rng(seed)
    return np.clip(np.rint(img + rng.normal(0.0, noise_sigma, img.shape)), 0, 255).astype(np.uint8), depth


def room_sequence(seed: int = 0, n_frames: int = 1000, w: int = BASE_W, h: int = BASE_H, fps: float = 30.0,
                  speed: float = 0.5, noise_sigma: float = 2.0, workers: int = 1, keep_depths: bool = False):
    """(RoomSequence, frames uint8 (n, h, w)).  Rendering takes a while at 640x480: pass
    `workers` > 1 to render in a process pool (created with the spawn method)."""
    rng = np.random.default_rng(seed)
    intr = Intrinsics.for_size(w, h)
    patches = make_room(rng)
    poses = room_path(rng, n_frames, fps, speed)
    jobs = [(patches, intr, w, h, poses[i], seed * 100003 + i, noise_sigma) for i in range(n_frames)]
    if workers > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            res = pool.map(_render_u8, jobs, chunksize=4)
    else:
        res = [_render_u8(j) for j in jobs]
    frames = np.stack([r[0] for r in res])
    depths = np.stack([r[1].astype(np.float32) for r in res]) if keep_depths else None
    return RoomSequence(w, h, intr, fps, patches, poses, res[0][1], depths), frames
