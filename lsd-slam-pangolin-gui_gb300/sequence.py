"""A minimal keyframe SLAM loop over the C-ABI, for full synthetic sequence runs.

The reference's SlamSystem (tracking, mapping and constraint-search threads, the g2o keyframe graph)
is absent from the reference tree; this driver strings the GPU path together the way those threads
use it, single-threaded and without relocalisation or loop-closure search beyond the candidates:

* tracking: every frame is aligned to the current keyframe (SE3Tracker::trackFrame, constant-
  velocity initial guess);
* mapping: every tracked frame updates the keyframe's depth (DepthMap::updateKeyframe, 8-bit
  frames), the tracking reference is refreshed from the smoothed depth every few frames, and after
  `kf_dist` metres of travel, a 6 degree turn, or when less than 55 % of the keyframe's points stay
  in view, the frame becomes the new keyframe (DepthMap::createKeyFrame: propagation +
  regularisation);
* constraint search: each new keyframe is aligned with Sim3Tracker::trackFrameSim3 to up to
  `n_candidates` earlier keyframes (the predecessor and the nearest others), all in one batched
  launch from device-resident keyframes; consistent results become pose-graph edges weighted with
  the tracker's 7x7 information;
* the keyframe poses are optimised by posegraph.PoseGraph (damped Gauss-Newton on Sim3).

The first keyframe is bootstrapped from the synthetic depth of frame 0 (5 % noise on textured
pixels); the reference initialises its first map randomly, which a synthetic run does not need.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

import lsdg
import posegraph as G
import synth


def _to4(T34):
    T = np.eye(4)
    T[:3, :] = np.asarray(T34, np.float64).reshape(3, 4)
    return T


def _hess7(stats):
    H = np.zeros((7, 7))
    q = 0
    for i in range(7):
        for j in range(i, 7):
            H[i, j] = H[j, i] = stats.hessian[q]
            q += 1
    return H


def _hess6(stats):
    H = np.zeros((6, 6))
    q = 0
    for i in range(6):
        for j in range(i, 6):
            H[i, j] = H[j, i] = stats.hessian[q]
            q += 1
    return H


@dataclasses.dataclass
class Keyframe:
    index: int          # frame index it was made from
    node: int           # pose-graph node
    frame: object       # lsdg.Frame with depth (tracking / Sim3 reference)


class SlamDriver:
    def __init__(self, ctx, w, h, intr, kf_dist=0.1, n_candidates=10, cand_radius=1.2, refresh_every=4,
                 min_update_baseline=0.0, reference="smoothed", min_validity=0):
        self.ctx, self.w, self.h, self.intr = ctx, w, h, intr
        self.reference = reference          # tracking reference depth: "smoothed" or "raw" filter state
        self.min_validity = min_validity    # pixels need this validity count to enter the reference
        self.min_update_baseline = min_update_baseline   # skip depth updates from frames closer than this
        self.kf_dist, self.n_candidates, self.cand_radius, self.refresh_every = kf_dist, n_candidates, cand_radius, refresh_every
        self.dm = lsdg.DepthMap(ctx, w, h, intr)
        self.tracker = lsdg.SE3Tracker(ctx)
        self.graph = G.PoseGraph()
        self.keyframes = []
        self.traj = []          # per frame: (keyframe number, frame-to-keyframe 4x4)
        self.lost = 0
        self.sim3_edges = 0
        self.sim3_rejected = 0
        self._batches = {}
        self._since_refresh = 0
        self._pool = [lsdg.Frame(ctx, w, h, intr) for _ in range(2)]   # tracking frames, reused
        self._pool_next = 0
        self.on_keyframe = None   # optional hook(frame index, smoothed inverse depth) for diagnostics
        self.optimize_every = 5   # pose-graph solve after this many keyframes with a non-sequential edge
        self.kf_angle = np.radians(6.0)   # ... or when the view turned this much
        self.kf_min_usage = 0.55          # ... or when fewer keyframe points than this stay in view
        self._loops_pending = 0

    # -- helpers ------------------------------------------------------------------------------
    def _reference_depth(self):
        if self.reference == "raw":
            st = self.dm.get(planes=("idepth", "var", "validity"))
            d, v = st["idepth"], st["var"]
        else:
            st = self.dm.get(planes=("idepth_smoothed", "var_smoothed", "validity"))
            d, v = st["idepth_smoothed"], st["var_smoothed"]
        if self.min_validity > 0 and self.keyframes:   # the bootstrap keyframe has no history yet
            d = np.where(st["validity"] >= self.min_validity, d, np.float32(-1))
        return d, v

    def _kf_frame(self, image_u8, k=0):
        d, v = self._reference_depth()
        if self.on_keyframe:
            self.on_keyframe(k, d)
        return lsdg.Frame(self.ctx, self.w, self.h, self.intr).upload(image_u8).set_depth(d, v)

    def _refresh(self, image_u8):
        d, v = self._reference_depth()
        self.keyframes[-1].frame.set_depth(d, v)

    def _batch(self, n):
        if n not in self._batches:
            self._batches[n] = lsdg.Batch(self.ctx, [self.w] * n, [self.h] * n, [self.intr] * n, sim3=True)
        return self._batches[n]

    # -- the loop -----------------------------------------------------------------------------
    def bootstrap(self, image_u8, idepth, idepth_var):
        self.dm.set_keyframe(image_u8.astype(np.float32), idepth, idepth_var)
        node = self.graph.add_node(np.eye(4))
        self.keyframes.append(Keyframe(0, node, self._kf_frame(image_u8)))
        self.traj.append((0, np.eye(4)))
        self._image = image_u8

    def step(self, k, image_u8):
        kf = self.keyframes[-1]
        # constant-velocity guess in the keyframe's frame
        c1 = self.traj[-1][1] if self.traj[-1][0] == len(self.keyframes) - 1 else np.eye(4)
        c0 = self.traj[-2][1] if len(self.traj) > 1 and self.traj[-2][0] == len(self.keyframes) - 1 else c1
        guess = c1 @ G.sim3_inv(c0) @ c1
        if not np.all(np.isfinite(guess)):
            guess = c1
        frame = self._pool[self._pool_next].upload(image_u8)
        self._pool_next ^= 1
        T, st = self.tracker.trackFrame(kf.frame, frame, guess[:3])
        f2k = _to4(T)
        if st.status != 0 or not np.all(np.isfinite(f2k)) or np.linalg.norm(f2k[:3, 3] - guess[:3, 3]) > 0.2:
            self.lost += 1
            f2k = guess
            st.status = 2
        self.traj.append((len(self.keyframes) - 1, f2k))
        key_to_frame = G.sim3_inv(f2k)
        if st.status == 0 and np.linalg.norm(f2k[:3, 3]) >= self.min_update_baseline:
            self.dm.updateKeyframe_u8(np.ascontiguousarray(image_u8[None]), [key_to_frame[:3]])
            self._since_refresh += 1
            if self._since_refresh >= self.refresh_every:
                self._refresh(image_u8)
                self._since_refresh = 0
        if st.status == 0 and (np.linalg.norm(f2k[:3, 3]) > self.kf_dist
                               or np.linalg.norm(G.so3_log(f2k[:3, :3])) > self.kf_angle
                               or st.usage < self.kf_min_usage):
            self._new_keyframe(k, image_u8, f2k, st)

    def _new_keyframe(self, k, image_u8, f2k, st):
        prev = self.keyframes[-1]
        self.dm.createKeyFrame(image_u8.astype(np.float32), G.sim3_inv(f2k)[:3])
        T_prev = self.graph.poses[prev.node]
        node = self.graph.add_node(T_prev @ f2k)
        kf = Keyframe(k, node, self._kf_frame(image_u8, k))
        self.keyframes.append(kf)
        self.traj[-1] = (len(self.keyframes) - 1, np.eye(4))
        self._since_refresh = 0
        # odometry edge from the tracking chain (SE3; the scale is tied by a strong prior)
        H6 = _hess6(st)
        if np.all(np.isfinite(H6)) and np.max(np.diag(H6)) > 0:
            Om = np.zeros((7, 7))
            Om[:6, :6] = H6
            Om[6, 6] = float(np.max(np.diag(H6)))
            self.graph.add_edge(prev.node, node, f2k, Om * 1e-3)
        # constraint search: Sim3 against the predecessor and the nearest earlier keyframes
        T_new = self.graph.poses[node]
        others = []
        for c in self.keyframes[:-2]:
            d = np.linalg.norm(self.graph.poses[c.node][:3, 3] - T_new[:3, 3])
            if d < self.cand_radius:
                others.append((d, c))
        others.sort(key=lambda x: x[0])
        cands = [prev] + [c for _, c in others[:self.n_candidates - 1]]
        inits = np.stack([G.to13(G.sim3_inv(self.graph.poses[c.node]) @ T_new) for c in cands])
        b = self._batch(len(cands))
        b.load_frames([c.frame for c in cands], [kf.frame] * len(cands), inits)
        b.run()
        out, stats = b.read()
        loop = False
        for c, o, s, i0 in zip(cands, out, stats, inits):
            if not (np.all(np.isfinite(o)) and 0.5 < o[12] < 2.0):
                self.sim3_rejected += 1
                continue
            Z = G.from13(o)
            dz = G.sim3_log(G.sim3_inv(G.from13(i0)) @ Z)
            ok = (s.status == 0 and np.linalg.norm(dz[:3]) < 0.25 * max(1.0, np.linalg.norm(Z[:3, 3]))
                  and np.linalg.norm(dz[3:6]) < 0.15 and abs(dz[6]) < 0.1)
            if not ok:
                self.sim3_rejected += 1
                continue
            H7 = _hess7(s)
            if not np.all(np.isfinite(H7)):
                self.sim3_rejected += 1
                continue
            self.graph.add_edge(c.node, node, Z, H7 * 1e-3)
            self.sim3_edges += 1
            loop = loop or c is not prev
        if loop:
            self._loops_pending += 1
            if self._loops_pending >= self.optimize_every:
                self._optimize(5)
                self._loops_pending = 0

    def _optimize(self, iterations):
        keep = [p.copy() for p in self.graph.poses]
        self.graph.optimize(iterations)
        if not all(np.all(np.isfinite(p)) for p in self.graph.poses):
            self.graph.poses = keep

    def finish(self):
        self._optimize(20)
        poses = []
        for kfi, f2k in self.traj:
            poses.append(self.graph.poses[self.keyframes[kfi].node] @ f2k)
        for b in self._batches.values():
            b.close()
        for f in self._pool:
            f.close()
        self.dm.close()
        return np.stack(poses)


def bootstrap_depth(seq, seed=0, rel_noise=0.05, grad_thresh=5.0, image=None):
    """Inverse depth of frame 0 on textured pixels (5 % noise) and its variance."""
    rng = np.random.default_rng(seed + 99991)
    img = image.astype(np.float64)
    gx, gy = synth.central_gradient(img)
    sel = ((gx * gx + gy * gy) > grad_thresh * grad_thresh) & np.isfinite(seq.first_depth)
    truth = 1.0 / seq.first_depth
    idepth = np.full(img.shape, -1.0)
    idepth[sel] = truth[sel] * (1.0 + rel_noise * rng.normal(size=int(sel.sum())))
    var = np.where(sel, (rel_noise * truth) ** 2, -1.0)
    return idepth.astype(np.float32), var.astype(np.float32)


def run(ctx, seq, frames, n_frames=None, on_keyframe=None, **kw):
    """Run the driver over the first n_frames frames; returns a result dict (fps, ATE, counts)."""
    n = seq.n if n_frames is None else min(n_frames, seq.n)
    drv = SlamDriver(ctx, seq.w, seq.h, seq.intr, **kw)
    drv.on_keyframe = on_keyframe
    idepth, var = bootstrap_depth(seq, image=frames[0])
    t0 = time.perf_counter()
    drv.bootstrap(frames[0], idepth, var)
    for k in range(1, n):
        drv.step(k, frames[k])
    est = drv.finish()
    wall = time.perf_counter() - t0
    gt_c = seq.cam_to_world[:n, :, 3]
    est_c = est[:, :3, 3]
    finite = np.all(np.isfinite(est.reshape(n, -1)), axis=1)
    bad = np.nonzero(~finite)[0]
    ate, (s, R, t) = G.ate_rmse(est_c[finite], gt_c[finite]) if finite.sum() >= 3 else (float("nan"), (0, 0, 0))
    path = float(np.sum(np.linalg.norm(np.diff(gt_c, axis=0), axis=1)))
    return {"frames": n, "seconds": wall, "fps": n / wall, "keyframes": len(drv.keyframes),
            "sim3_edges": drv.sim3_edges, "sim3_rejected": drv.sim3_rejected, "lost_frames": drv.lost,
            "ate_rmse_m": ate, "path_m": path, "ate_over_path": ate / max(path, 1e-9), "alignment_scale": s,
            "non_finite_frames": int(len(bad)), "first_non_finite": int(bad[0]) if len(bad) else -1}
