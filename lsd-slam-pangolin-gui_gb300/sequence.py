"""Full synthetic sequence runs of the SLAM loop (lsdg_slam, csrc/slam.cu) and their evaluation.

The loop itself -- tracking and mapping of every frame, keyframes (refined before they are left, or an
earlier keyframe made current again), batched Sim3 constraint search in both directions on a worker
thread, the Sim3 pose graph -- is the library's C++ (lsdg_slam_*);
this module feeds it a rendered sequence the way the reference's InputThread feeds SlamSystem
(lib/App/InputThread.cpp:71), then scores the trajectory against the ground truth: absolute
trajectory error of the camera centres after the best similarity alignment (Umeyama 1991), as a
fraction of the path length.

The first keyframe is bootstrapped from the synthetic depth of frame 0 (5 % noise on textured
pixels); the reference initialises its first map randomly, which a synthetic run does not need.
"""
from __future__ import annotations

import time

import numpy as np

import lsdg
import synth


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


def umeyama(src, dst, with_scale=True):
    """Similarity (s, R, t) minimising sum |dst - (s R src + t)|^2 (Umeyama 1991)."""
    src, dst = np.asarray(src, np.float64), np.asarray(dst, np.float64)
    ms, md = src.mean(0), dst.mean(0)
    xs, xd = src - ms, dst - md
    C = xd.T @ xs / len(src)
    U, D, Vt = np.linalg.svd(C)
    S = np.eye(3)
    if np.linalg.det(U) * np.linalg.det(Vt) < 0:
        S[2, 2] = -1
    R = U @ S @ Vt
    s = float(np.trace(np.diag(D) @ S) / (xs ** 2).sum() * len(src)) if with_scale else 1.0
    return s, R, md - s * R @ ms


def ate_rmse(est_centres, gt_centres):
    """RMSE of camera centres after the best similarity alignment, and that alignment."""
    s, R, t = umeyama(est_centres, gt_centres)
    aligned = (s * (R @ np.asarray(est_centres, np.float64).T)).T + t
    return float(np.sqrt(np.mean(np.sum((aligned - gt_centres) ** 2, axis=1)))), (s, R, t)


def run(seq, frames, n_frames=None, params=None, slam_params=None, device=0, pose_file=None):
    """Feed the first n_frames frames to a fresh lsdg_slam; returns a result dict (fps, ATE, counts)."""
    n = seq.n if n_frames is None else min(n_frames, seq.n)
    sys_ = lsdg.SlamSystem(seq.w, seq.h, seq.intr, params=params, slam_params=slam_params, device=device)
    try:
        idepth, var = bootstrap_depth(seq, image=frames[0])
        t0 = time.perf_counter()
        sys_.bootstrap(0, frames[0], idepth, var)
        for k in range(1, n):
            sys_.nextImage(k, frames[k])
        sys_.finalize()
        wall = time.perf_counter() - t0
        poses = sys_.poses()
        stats = sys_.stats()
        graph = sys_.keyframe_graph()
        if pose_file:
            sys_.write_pose_file(pose_file)
    finally:
        sys_.close()
    est_c = poses[:, 9:12]
    gt_c = seq.cam_to_world[:n, :, 3]
    finite = np.all(np.isfinite(poses), axis=1)
    bad = np.nonzero(~finite)[0]
    ate, (s, _, _) = ate_rmse(est_c[finite], gt_c[finite]) if finite.sum() >= 3 else (float("nan"), (0.0, 0, 0))
    path = float(np.sum(np.linalg.norm(np.diff(gt_c, axis=0), axis=1)))
    # the ground truth's own RMS spread about its centroid: a trajectory collapsed to its mean scores
    # this ATE, so the ATE means something only well below it
    spread = float(np.sqrt(np.mean(np.sum((gt_c - gt_c.mean(0)) ** 2, axis=1))))
    return {"frames": n, "seconds": wall, "fps": n / wall, "keyframes": stats["keyframes"],
            "sim3_edges": stats["sim3_edges"], "sim3_rejected": stats["sim3_rejected"],
            "lost_frames": stats["lost_frames"], "graph_optimisations": stats["graph_optimisations"],
            "reactivations": stats["reactivations"],
            "keyframe_graph_nodes": len(graph), "ate_rmse_m": ate, "path_m": path,
            "ate_over_path": ate / max(path, 1e-9), "gt_spread_m": spread, "ate_over_gt_spread": ate / max(spread, 1e-9),
            "alignment_scale": s,
            "non_finite_frames": int(len(bad)), "first_non_finite": int(bad[0]) if len(bad) else -1}
