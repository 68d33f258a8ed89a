"""A small Sim3 pose graph (keyframe poses, Sim3 constraints) solved by damped Gauss-Newton.

The reference keeps its keyframe graph in g2o (KeyFrameGraph, absent from the reference tree;
PangolinOutputIOWrapper::publishKeyframeGraph, lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:148-168
shows the interface it feeds the viewer).  This is the project's own stand-in for full sequence
runs: nodes are camera-to-world Sim3 poses, an edge (i, j, Z, Omega) says "pose j seen from pose
i is Z" with information Omega (7x7 in the twist order v, omega, log-scale), and the cost is
sum rho(r^T Omega r) with r = log(Z^-1 T_i^-1 T_j) and a Huber kernel rho on the Mahalanobis norm.  Perturbations are on the right (T <- T exp(d));
to first order r(d) = r + d_j - Adj(T_j^-1 T_i) d_i.  A few hundred nodes make a dense solve cheap.

Sim3 poses here are 4x4 numpy matrices [[s R, t], [0, 1]].
"""
from __future__ import annotations

import math

import numpy as np

_GL_X, _GL_W = np.polynomial.legendre.leggauss(16)
_GL_T = 0.5 * (_GL_X + 1.0)   # nodes on [0, 1]
_GL_W = 0.5 * _GL_W


def hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def so3_exp(w):
    th = float(np.linalg.norm(w))
    K = hat(w)
    if th < 1e-8:
        return np.eye(3) + K + 0.5 * K @ K
    return np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / (th * th) * K @ K


def so3_log(R):
    c = max(-1.0, min(1.0, (np.trace(R) - 1.0) / 2.0))
    th = math.acos(c)
    W = (R - R.T) / 2.0
    w = np.array([W[2, 1], W[0, 2], W[1, 0]])
    if th < 1e-6:
        return w
    if math.pi - th < 1e-4:
        # near pi: axis from the symmetric part
        B = (R + np.eye(3)) / 2.0
        k = int(np.argmax(np.diag(B)))
        axis = B[:, k] / math.sqrt(max(B[k, k], 1e-300))
        axis = axis if np.dot(axis, w) >= 0 else -axis
        return axis * th
    return w * th / math.sin(th)


def _V_quadrature(w, sigma):
    """V = int_0^1 e^(sigma tau) R(tau w) dtau by 16-point Gauss-Legendre (reference form)."""
    V = np.zeros((3, 3))
    for t, wt in zip(_GL_T, _GL_W):
        V += wt * math.exp(sigma * t) * so3_exp(t * np.asarray(w))
    return V


def _V(w, sigma):
    """V = a0 I + a1 K + a2 K^2 (K = hat(w)) with a0 = int e^(s t), a1 = int e^(s t) sin(th t)/th,
    a2 = int e^(s t) (1 - cos(th t))/th^2 over [0, 1]: closed forms, series where they cancel."""
    th2 = float(np.dot(w, w))
    th = math.sqrt(th2)
    s = float(sigma)
    if abs(s) < 1e-5:
        a0 = 1.0 + s / 2.0 + s * s / 6.0
    else:
        a0 = math.expm1(s) / s
    if th < 1e-3:
        # theta series with I_n = int t^(n-1) e^(s t): a1 = I_2 - th^2 I_4 / 6, a2 = I_3 / 2 - th^2 I_5 / 24
        if abs(s) < 1e-3:
            I = [None, 1.0, 0.5 + s / 3.0, 1 / 3.0 + s / 4.0, 0.25 + s / 5.0, 0.2 + s / 6.0]
        else:
            es = math.exp(s)
            I = [None, math.expm1(s) / s]
            for n in range(2, 6):
                I.append((es - (n - 1) * I[-1]) / s)
        a1 = I[2] - th2 * I[4] / 6.0
        a2 = I[3] / 2.0 - th2 * I[5] / 24.0
    else:
        es = math.exp(s)
        D = s * s + th2
        S1 = (es * (s * math.sin(th) - th * math.cos(th)) + th) / D
        C1 = (es * (s * math.cos(th) + th * math.sin(th)) - s) / D
        a1 = S1 / th
        a2 = (a0 - C1) / th2
    K = hat(w)
    return a0 * np.eye(3) + a1 * K + a2 * (K @ K)


def sim3_exp(xi):
    v, w, sigma = np.asarray(xi[:3]), np.asarray(xi[3:6]), float(xi[6])
    T = np.eye(4)
    T[:3, :3] = math.exp(sigma) * so3_exp(w)
    T[:3, 3] = _V(w, sigma) @ v
    return T


def sim3_log(T):
    M = T[:3, :3]
    s = float(np.cbrt(np.linalg.det(M)))
    R = M / s
    w = so3_log(R)
    sigma = math.log(s)
    v = np.linalg.solve(_V(w, sigma), T[:3, 3])
    return np.concatenate([v, w, [sigma]])


def sim3_inv(T):
    M = T[:3, :3]
    s2 = float(np.dot(M[0], M[0]))
    Mi = M.T / s2
    out = np.eye(4)
    out[:3, :3] = Mi
    out[:3, 3] = -Mi @ T[:3, 3]
    return out


def adjoint(T):
    """Adj(T) of a Sim3 [[s R, t], [0, 1]] on twists (v, omega, sigma)."""
    M = T[:3, :3]
    s = float(np.cbrt(np.linalg.det(M)))
    R = M / s
    t = T[:3, 3]
    A = np.zeros((7, 7))
    A[:3, :3] = s * R
    A[:3, 3:6] = hat(t) @ R
    A[:3, 6] = -t
    A[3:6, 3:6] = R
    A[6, 6] = 1.0
    return A


def from13(p):
    p = np.asarray(p, np.float64).reshape(-1)
    T = np.eye(4)
    T[:3, :3] = p[12] * p[:9].reshape(3, 3)
    T[:3, 3] = p[9:12]
    return T


def to13(T):
    M = T[:3, :3]
    s = float(np.cbrt(np.linalg.det(M)))
    return np.concatenate([(M / s).ravel(), T[:3, 3], [s]])


class PoseGraph:
    def __init__(self):
        self.poses = []      # 4x4 camera-to-world Sim3
        self.edges = []      # (i, j, Z 4x4, Omega 7x7)
        self.fixed = {0}

    def add_node(self, T) -> int:
        self.poses.append(np.array(T, np.float64))
        return len(self.poses) - 1

    def add_edge(self, i: int, j: int, Z, omega):
        self.edges.append((i, j, np.array(Z, np.float64), np.array(omega, np.float64)))

    def residual(self, e):
        i, j, Z, _ = e
        return sim3_log(sim3_inv(Z) @ sim3_inv(self.poses[i]) @ self.poses[j])

    huber = 3.0  # robust kernel on the Mahalanobis norm of an edge residual (in sigmas)

    def _weight(self, r, Om):
        m2 = float(r @ Om @ r)
        m = math.sqrt(max(m2, 0.0))
        return 1.0 if m <= self.huber else self.huber / m

    def _edge_cost(self, r, Om):
        m2 = float(r @ Om @ r)
        m = math.sqrt(max(m2, 0.0))
        return m2 if m <= self.huber else self.huber * (2.0 * m - self.huber)

    def cost(self) -> float:
        return float(sum(self._edge_cost(self.residual(e), e[3]) for e in self.edges))

    def optimize(self, iterations: int = 10, lam: float = 1e-4):
        """Damped Gauss-Newton with the first node (and any in `fixed`) held; returns the final cost."""
        n = len(self.poses)
        free = [k for k in range(n) if k not in self.fixed]
        col = {k: 7 * q for q, k in enumerate(free)}
        m = 7 * len(free)
        if m == 0 or not self.edges:
            return self.cost()
        cost = self.cost()
        for _ in range(iterations):
            H = np.zeros((m, m))
            b = np.zeros(m)
            for e in self.edges:
                i, j, _, Om0 = e
                r = self.residual(e)
                Om = self._weight(r, Om0) * Om0   # iteratively reweighted (Huber)
                Ji = -adjoint(sim3_inv(self.poses[j]) @ self.poses[i])
                blocks = []
                if i in col:
                    blocks.append((col[i], Ji))
                if j in col:
                    blocks.append((col[j], np.eye(7)))
                for ca, Ja in blocks:
                    b[ca:ca + 7] += Ja.T @ Om @ r
                    for cb, Jb in blocks:
                        H[ca:ca + 7, cb:cb + 7] += Ja.T @ Om @ Jb
            while True:
                d = np.linalg.solve(H + lam * np.diag(np.maximum(np.diag(H), 1e-12)), -b)
                old = [p.copy() for p in self.poses]
                for k in free:
                    self.poses[k] = self.poses[k] @ sim3_exp(d[col[k]:col[k] + 7])
                new = self.cost()
                if new <= cost:
                    lam = max(lam * 0.3, 1e-9)
                    break
                self.poses = old
                lam *= 10
                if lam > 1e8:
                    return cost
            if cost - new < 1e-10 * max(cost, 1e-30):
                cost = new
                break
            cost = new
        return cost


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
    t = md - s * R @ ms
    return s, R, t


def ate_rmse(est_centres, gt_centres, with_scale=True):
    """Absolute trajectory error (RMSE of camera centres) after the best similarity alignment."""
    s, R, t = umeyama(est_centres, gt_centres, with_scale)
    aligned = (s * (R @ np.asarray(est_centres, np.float64).T)).T + t
    return float(np.sqrt(np.mean(np.sum((aligned - gt_centres) ** 2, axis=1)))), (s, R, t)
