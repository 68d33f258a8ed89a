"""Second, independent restatement (numpy float32, vectorised) of the pyramid and keyframe-point
construction, used to pin the C++ oracle: numpy float32 arithmetic rounds each operation like
the oracle does, so both must agree bit for bit."""
import numpy as np


def pyramid(img: np.ndarray, levels: int):
    I = img.astype(np.float32)
    out = []
    for l in range(levels):
        if l > 0:
            P = out[-1][..., 0]
            I = ((P[0::2, 0::2] + P[0::2, 1::2]) + (P[1::2, 0::2] + P[1::2, 1::2])) * np.float32(0.25)
        h, w = I.shape
        gx = np.zeros_like(I)
        gy = np.zeros_like(I)
        gx[:, 1:-1] = (I[:, 2:] - I[:, :-2]) * np.float32(0.5)
        gy[1:-1, :] = (I[2:, :] - I[:-2, :]) * np.float32(0.5)
        out.append(np.stack([I, gx, gy, np.zeros_like(I)], axis=-1))
    return out


def depth_pyramid(idepth: np.ndarray, var: np.ndarray, levels: int):
    d = idepth.astype(np.float32).copy()
    v = var.astype(np.float32).copy()
    ok = (d > 0) & (v > 0)
    d[~ok] = -1
    v[~ok] = -1
    D, V = [d], [v]
    for l in range(1, levels):
        pd, pv = D[-1], V[-1]
        h, w = pd.shape[0] // 2, pd.shape[1] // 2
        sw = np.zeros((h, w), np.float32)
        swd = np.zeros((h, w), np.float32)
        n = np.zeros((h, w), np.int32)
        for (dy, dx) in ((0, 0), (0, 1), (1, 0), (1, 1)):
            cd = pd[dy::2, dx::2]
            cv = pv[dy::2, dx::2]
            m = (cd > 0) & (cv > 0)
            with np.errstate(divide="ignore"):
                wt = np.where(m, np.float32(1) / np.where(m, cv, np.float32(1)), np.float32(0)).astype(np.float32)
            sw = np.where(m, sw + wt, sw).astype(np.float32)
            swd = np.where(m, swd + wt * cd, swd).astype(np.float32)
            n += m
        valid = n > 0
        with np.errstate(divide="ignore", invalid="ignore"):
            nd = np.where(valid, swd / np.where(valid, sw, 1), -1).astype(np.float32)
            nv = np.where(valid, n.astype(np.float32) / np.where(valid, sw, 1), -1).astype(np.float32)
        D.append(nd)
        V.append(nv)
    return D, V


def level_intrinsics(fx, fy, cx, cy, levels):
    out = []
    for l in range(levels):
        out.append((fx, fy, cx, cy))
        fx, fy = fx * 0.5, fy * 0.5
        cx = (cx + 0.5) * 0.5 - 0.5
        cy = (cy + 0.5) * 0.5 - 0.5
    return out


def points(I_levels, D, V, intr, levels):
    cams = level_intrinsics(*intr, levels)
    res = []
    for l in range(levels):
        fx, fy, cx, cy = cams[l]
        d, v = D[l], V[l]
        ys, xs = np.nonzero((d > 0) & (v > 0))
        z = np.float32(1) / d[ys, xs]
        X = ((xs.astype(np.float32) - np.float32(cx)) * np.float32(1.0 / fx)) * z
        Y = ((ys.astype(np.float32) - np.float32(cy)) * np.float32(1.0 / fy)) * z
        Ik = I_levels[l][ys, xs, 0]
        res.append((np.stack([X, Y, z, Ik], axis=1).astype(np.float32), v[ys, xs]))
    return res
