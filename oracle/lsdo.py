"""ctypes wrapper of the CPU ORACLE (oracle/liblsdo.so).  Test infrastructure only: imported by
tests/, the smoke check and bench.py's cpu_baseline leg, never by the product package."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "lsd-slam-pangolin-gui_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
import lsdg_types as T  # noqa: E402

_lib = None
_fast_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def lib():
    """The parity oracle (oracle/liblsdo.so: no FMA contraction, the kernels' operation order)."""
    global _lib
    if _lib is None:
        sys.path.insert(0, HERE)
        import build as _b  # oracle/build.py
        _lib = _bind(C.CDLL(_b.build()))
    return _lib


def fast_lib():
    """The same restatement built for speed (oracle/liblsdo_fast.so: -O3, FMA contraction, the
    host CPU's instruction set named explicitly): the timed CPU baseline.  Its results are checked
    against the FP64 oracle by tolerance, never used as the parity reference."""
    global _fast_lib
    if _fast_lib is None:
        sys.path.insert(0, HERE)
        import build as _b  # oracle/build.py
        _fast_lib = _bind(C.CDLL(_b.build_fast()))
    return _fast_lib


def fast_build_flags() -> str:
    sys.path.insert(0, HERE)
    import build as _b  # oracle/build.py
    fast_lib()
    return " ".join(_b.fast_flags_used())


def _bind(L):
    """ctypes signatures of the oracle's entry points."""
    L.lsdo_default_params.argtypes = [C.POINTER(T.Params)]
    L.lsdo_pyramid_f.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f32p]
    L.lsdo_pyramid_d.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f64p]
    L.lsdo_keyframe_f.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.c_int,
                                  _f32p, _f32p, _f32p, _f32p, C.c_int, _i32p]
    L.lsdo_keyframe_f.restype = C.c_int
    for nm in ("lsdo_se3_normal_equations_f", "lsdo_se3_normal_equations_d"):
        f = getattr(L, nm)
        f.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                      C.POINTER(T.Params), C.c_int, _f64p, _f64p]
        f.restype = C.c_int
    for nm in ("lsdo_track_se3_f", "lsdo_track_se3_d"):
        f = getattr(L, nm)
        f.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                      C.POINTER(T.Params), _f64p, _f64p, C.POINTER(T.TrackStats), C.c_int]
        f.restype = C.c_int
    L.lsdo_se3_fixed_energy_d.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                          C.POINTER(T.Params), C.c_int, _f64p, _f64p, _f64p]
    L.lsdo_se3_fixed_energy_d.restype = C.c_int
    L.lsdo_track_trace.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                   C.POINTER(T.Params), _f64p, _f64p, C.POINTER(T.TrackStats), _f64p, C.c_int,
                                   C.POINTER(C.c_int)]
    L.lsdo_track_trace.restype = C.c_int
    for nm in ("lsdo_track_batch_f", "lsdo_track_batch_d"):
        f = getattr(L, nm)
        f.argtypes = [C.c_int, _i32p, _i32p, C.POINTER(T.Intrinsics), _f32p, _f32p, _f32p,
                      _f32p, _f64p, _f64p, C.POINTER(T.TrackStats), C.POINTER(T.Params), C.c_int]
        f.restype = C.c_int
    for nm in ("lsdo_depth_pipeline_f", "lsdo_depth_pipeline_d"):
        f = getattr(L, nm)
        f.argtypes = [C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.POINTER(T.Params), _f32p, _f32p, _f32p, C.c_int,
                      _f32p, _f64p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        f.restype = C.c_int
    L.lsdo_sim3_normal_equations.argtypes = [C.c_int] + [_f32p] * 6 + [C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                                                         C.POINTER(T.Params), C.c_int, _f64p, _f64p]
    L.lsdo_sim3_normal_equations.restype = C.c_int
    L.lsdo_track_sim3.argtypes = [C.c_int] + [_f32p] * 6 + [C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                                            C.POINTER(T.Params), _f64p, _f64p, C.POINTER(T.TrackStats)]
    L.lsdo_track_sim3.restype = C.c_int
    L.lsdo_sim3_exp.argtypes = [_f64p, _f64p]
    _vp = C.c_void_p
    L.lsdo_energy_points.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                     C.POINTER(T.Params), C.c_int, _vp, _vp]
    L.lsdo_energy_points.restype = C.c_int
    L.lsdo_energy.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                              C.POINTER(T.Params), C.c_int, _f64p, C.c_int] + [_vp] * 8 + \
                             [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.lsdo_energy.restype = C.c_int
    L.lsdo_energy_refine.argtypes = [C.c_int, _f32p, _f32p, _f32p, C.c_int, _f32p, C.c_int, C.c_int,
                                     C.POINTER(T.Intrinsics), C.POINTER(T.Params), C.c_int, _f64p, C.c_int, _vp,
                                     _f32p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_long),
                                     C.c_int]
    L.lsdo_energy_refine.restype = C.c_int
    L.lsdo_cloud_build.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                   _vp, _vp, _vp]
    L.lsdo_cloud_build.restype = C.c_int
    L.lsdo_undistort_map.argtypes = [C.POINTER(T.Calibration), C.c_int, C.c_int, C.POINTER(T.Intrinsics), _f32p]
    L.lsdo_undistort.argtypes = [_vp, C.c_int, C.c_int, _f32p, C.c_int, _vp]
    L.lsdo_hardware_threads.restype = C.c_int
    L.lsdo_depth_trace.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.POINTER(T.Params), _f32p,
                                   _f32p, _f32p, C.c_int, _f32p, _f64p, C.c_void_p, C.c_void_p, C.c_int,
                                   np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS"), C.c_void_p, C.c_long]
    L.lsdo_depth_trace.restype = C.c_long
    return L


def default_params() -> T.Params:
    p = T.Params()
    lib().lsdo_default_params(C.byref(p))
    return p


def _intr(intr) -> T.Intrinsics:
    if isinstance(intr, T.Intrinsics):
        return intr
    fx, fy, cx, cy = intr.as_tuple() if hasattr(intr, "as_tuple") else intr
    return T.Intrinsics(fx, fy, cx, cy)


def level_sizes(w, h, levels):
    return [(w >> l, h >> l) for l in range(levels)]


def pyramid(img: np.ndarray, levels: int = 5, double: bool = False):
    """List of float4 {I, gx, gy, 0} arrays [h_l, w_l, 4]."""
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape
    sizes = level_sizes(w, h, levels)
    n = sum(a * b for a, b in sizes)
    out = np.zeros(4 * n, np.float64 if double else np.float32)
    (lib().lsdo_pyramid_d if double else lib().lsdo_pyramid_f)(img, w, h, levels, out)
    res, off = [], 0
    for (a, b) in sizes:
        res.append(out[off:off + 4 * a * b].reshape(b, a, 4))
        off += 4 * a * b
    return res


def keyframe(img, idepth, var, intr, levels: int = 5):
    """Depth pyramid and reference points (float oracle).  Returns (depth[l], var[l], xyzi[l], pvar[l])."""
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape
    sizes = level_sizes(w, h, levels)
    n = sum(a * b for a, b in sizes)
    d = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    xyzi = np.zeros(4 * n, np.float32)
    pv = np.zeros(n, np.float32)
    counts = np.zeros(levels, np.int32)
    k = _intr(intr)
    rc = lib().lsdo_keyframe_f(img, np.ascontiguousarray(idepth, np.float32), np.ascontiguousarray(var, np.float32),
                               w, h, C.byref(k), levels, d, v, xyzi, pv, n, counts)
    assert rc == 0
    D, V, P, PV = [], [], [], []
    off = 0
    poff = 0
    for l, (a, b) in enumerate(sizes):
        D.append(d[off:off + a * b].reshape(b, a))
        V.append(v[off:off + a * b].reshape(b, a))
        off += a * b
        c = int(counts[l])
        P.append(xyzi[4 * poff:4 * (poff + c)].reshape(c, 4))
        PV.append(pv[poff:poff + c])
        poff += c
    return D, V, P, PV


def se3_normal_equations(pair, ref_to_frame: np.ndarray, level: int, params: T.Params = None, double: bool = False):
    p = params or default_params()
    out = np.zeros(T.NE_SIZE, np.float64)
    f = lib().lsdo_se3_normal_equations_d if double else lib().lsdo_se3_normal_equations_f
    rc = f(pair.ref_image, pair.ref_idepth, pair.ref_idepth_var, pair.new_image, pair.w, pair.h,
           C.byref(_intr(pair.intr)), C.byref(p), level, np.ascontiguousarray(ref_to_frame, np.float64).ravel(), out)
    assert rc == 0
    return out


def se3_fixed_energy(pair, T_fix, T_eval, level, params=None):
    """FP64 sums at T_eval with variances and participating points fixed by a first pass at T_fix."""
    p = params or default_params()
    out = np.zeros(T.NE_SIZE, np.float64)
    rc = lib().lsdo_se3_fixed_energy_d(pair.ref_image, pair.ref_idepth, pair.ref_idepth_var, pair.new_image, pair.w,
                                       pair.h, C.byref(_intr(pair.intr)), C.byref(p), level,
                                       np.ascontiguousarray(T_fix, np.float64).ravel(),
                                       np.ascontiguousarray(T_eval, np.float64).ravel(), out)
    assert rc == 0
    return out


def track_se3(pair, init: np.ndarray = None, params: T.Params = None, double: bool = False, threads: int = 1):
    p = params or default_params()
    init = np.eye(3, 4) if init is None else init
    out = np.zeros(12, np.float64)
    st = T.TrackStats()
    f = lib().lsdo_track_se3_d if double else lib().lsdo_track_se3_f
    rc = f(pair.ref_image, pair.ref_idepth, pair.ref_idepth_var, pair.new_image, pair.w, pair.h,
           C.byref(_intr(pair.intr)), C.byref(p), np.ascontiguousarray(init, np.float64).ravel(), out, C.byref(st), threads)
    return rc, out.reshape(3, 4), st


def track_trace(pair, init=None, params=None, double=False):
    """trackFrame with a per-pass trace: rows {level, iteration, lambda, accepted (2 = convergence
    test), mean energy, points, max |undamped step|, 0}."""
    p = params or default_params()
    init = np.eye(3, 4) if init is None else init
    out = np.zeros(12, np.float64)
    st = T.TrackStats()
    buf = np.zeros(8 * 4096, np.float64)
    n = C.c_int()
    rc = lib().lsdo_track_trace(int(double), pair.ref_image, pair.ref_idepth, pair.ref_idepth_var, pair.new_image,
                                pair.w, pair.h, C.byref(_intr(pair.intr)), C.byref(p),
                                np.ascontiguousarray(init, np.float64).ravel(), out, C.byref(st), buf, buf.size, C.byref(n))
    return rc, out.reshape(3, 4), st, buf[:8 * n.value].reshape(-1, 8)


def track_batch(pairs, inits=None, params: T.Params = None, threads: int = None, double: bool = False,
                fast: bool = False):
    """The batched workload on the CPU, pairs spread over threads: float (the CPU baseline; `fast`
    selects the speed build) or double (the FP64 oracle of the whole batch)."""
    p = params or default_params()
    n = len(pairs)
    threads = threads or hardware_threads()
    widths = np.array([q.w for q in pairs], np.int32)
    heights = np.array([q.h for q in pairs], np.int32)
    intr = (T.Intrinsics * n)(*[_intr(q.intr) for q in pairs])
    cat = lambda name: np.ascontiguousarray(np.concatenate([getattr(q, name).ravel() for q in pairs]), np.float32)
    init = np.concatenate([np.eye(3, 4).ravel() for _ in range(n)]) if inits is None else np.ascontiguousarray(inits, np.float64).ravel()
    out = np.zeros(12 * n, np.float64)
    stats = (T.TrackStats * n)()
    L = fast_lib() if fast else lib()
    f = L.lsdo_track_batch_d if double else L.lsdo_track_batch_f
    f(n, widths, heights, intr, cat("ref_image"), cat("ref_idepth"), cat("ref_idepth_var"),
      cat("new_image"), init, out, stats, C.byref(p), threads)
    return out.reshape(n, 3, 4), stats


def hardware_threads() -> int:
    return int(lib().lsdo_hardware_threads())


DEPTH_PLANES = ("idepth", "var", "idepth_smoothed", "var_smoothed", "validity", "blacklist")


def _planes(buf, h, w):
    n = h * w
    out = {}
    for k, name in enumerate(DEPTH_PLANES):
        a = buf[k * n:(k + 1) * n].reshape(h, w)
        out[name] = a.astype(np.int32) if name in ("validity", "blacklist") else a
    return out


def depth_pipeline(seq, params=None, double=False, regularize=True, propagate=True, n_refs=None, threads=1,
                   init_idepth=None, init_var=None, fast=False):
    """DepthMap::updateKeyframe over the sequence's references (+ regularize), then createKeyFrame
    (propagate + regularize) into the next frame.  Returns (after_update, after_propagate) dicts."""
    p = params or default_params()
    h, w = seq.h, seq.w
    n = len(seq.ref_images) if n_refs is None else n_refs
    refs = np.ascontiguousarray(np.concatenate([r.ravel() for r in seq.ref_images[:n]]), np.float32)
    poses = np.concatenate([np.ascontiguousarray(_inv(T_), np.float64).ravel() for T_ in seq.ref_frame_to_key[:n]])
    upd = np.zeros(6 * h * w, np.float32)
    prop = np.zeros(6 * h * w, np.float32) if propagate else None
    nimg = np.ascontiguousarray(seq.next_image, np.float32) if propagate else None
    knew = np.ascontiguousarray(_inv(seq.next_to_key), np.float64).ravel() if propagate else None
    flags = (1 if regularize else 0) | (2 if regularize else 0)
    L = fast_lib() if fast else lib()
    f = L.lsdo_depth_pipeline_d if double else L.lsdo_depth_pipeline_f
    d0 = seq.init_idepth if init_idepth is None else init_idepth
    v0 = seq.init_var if init_var is None else init_var
    f(w, h, C.byref(_intr(seq.intr)), C.byref(p), np.ascontiguousarray(seq.key_image, np.float32),
      np.ascontiguousarray(d0, np.float32), np.ascontiguousarray(v0, np.float32), n, refs, poses,
      nimg.ctypes.data if propagate else None, knew.ctypes.data if propagate else None, flags,
      upd.ctypes.data, prop.ctypes.data if propagate else None, threads)
    return _planes(upd, h, w), (_planes(prop, h, w) if propagate else None)


# One record of the depth filter's decision trace (lsdo_depth.cpp, DecisionRec).
DECISION_DTYPE = np.dtype([("pixel", np.int32), ("stage", np.int32), ("ref", np.int32), ("id", np.int32),
                           ("outcome", np.int32), ("aux", np.int32), ("q", np.float64), ("thr", np.float64)])


def depth_trace(seq, mask, double=False, params=None, regularize=True, propagate=True, n_refs=None):
    """The depth_pipeline of `seq` with every threshold decision recorded, in execution order, for
    the pixels where mask[stage] is true: stage 0 observe, 1 the update's regularisation,
    2 propagation (keyed by the old keyframe pixel), 3 the new keyframe's regularisation.
    `mask` is bool [4, h, w]."""
    p = params or default_params()
    h, w = seq.h, seq.w
    n = len(seq.ref_images) if n_refs is None else n_refs
    refs = np.ascontiguousarray(np.concatenate([r.ravel() for r in seq.ref_images[:n]]), np.float32)
    poses = np.concatenate([np.ascontiguousarray(_inv(T_), np.float64).ravel() for T_ in seq.ref_frame_to_key[:n]])
    nimg = np.ascontiguousarray(seq.next_image, np.float32) if propagate else None
    knew = np.ascontiguousarray(_inv(seq.next_to_key), np.float64).ravel() if propagate else None
    flags = (1 if regularize else 0) | (2 if regularize else 0)
    m = np.ascontiguousarray(np.asarray(mask, bool).reshape(4, h * w), np.uint8).ravel()
    cap = 1 << 16
    while True:
        out = np.zeros(cap, DECISION_DTYPE)
        got = lib().lsdo_depth_trace(int(double), w, h, C.byref(_intr(seq.intr)), C.byref(p),
                                     np.ascontiguousarray(seq.key_image, np.float32),
                                     np.ascontiguousarray(seq.init_idepth, np.float32),
                                     np.ascontiguousarray(seq.init_var, np.float32), n, refs, poses,
                                     nimg.ctypes.data if propagate else None, knew.ctypes.data if propagate else None,
                                     flags, m, out.ctypes.data, cap)
        if got <= cap:
            return out[:got]
        cap = int(got)


def _inv(T_):
    R = T_[:, :3]
    t = T_[:, 3]
    out = np.zeros((3, 4))
    out[:, :3] = R.T
    out[:, 3] = -R.T @ t
    return out


def _sim3_inputs(pair):
    f = lambda a: np.ascontiguousarray(a, np.float32)
    return (f(pair.ref_image), f(pair.ref_idepth), f(pair.ref_idepth_var), f(pair.new_image), f(pair.new_idepth),
            f(pair.new_idepth_var))


def sim3_normal_equations(pair, ref_to_frame13, level, params=None, double=False):
    p = params or default_params()
    out = np.zeros(T.NE_SIZE_SIM3, np.float64)
    rc = lib().lsdo_sim3_normal_equations(int(double), *_sim3_inputs(pair), pair.w, pair.h, C.byref(_intr(pair.intr)),
                                          C.byref(p), level, np.ascontiguousarray(ref_to_frame13, np.float64), out)
    assert rc == 0
    return out


def track_sim3(pair, init13=None, params=None, double=False):
    p = params or default_params()
    init13 = np.concatenate([np.eye(3).ravel(), np.zeros(3), [1.0]]) if init13 is None else init13
    out = np.zeros(13, np.float64)
    st = T.TrackStats()
    rc = lib().lsdo_track_sim3(int(double), *_sim3_inputs(pair), pair.w, pair.h, C.byref(_intr(pair.intr)),
                               C.byref(p), np.ascontiguousarray(init13, np.float64), out, C.byref(st))
    return rc, out, st


def sim3_exp(xi):
    out = np.zeros(12, np.float64)
    lib().lsdo_sim3_exp(np.ascontiguousarray(xi, np.float64), out)
    return out.reshape(3, 4)


def sim3_error(a13, b13):
    """(rotation angle, translation distance, |scale ratio - 1|) between two 13-double Sim3 poses."""
    import synth
    A = np.zeros((3, 4)); A[:, :3] = np.reshape(a13[:9], (3, 3)); A[:, 3] = a13[9:12]
    B = np.zeros((3, 4)); B[:, :3] = np.reshape(b13[:9], (3, 3)); B[:, 3] = b13[9:12]
    ang, dist = synth.pose_error(A, B)
    return ang, dist, abs(a13[12] / b13[12] - 1.0)


# ------------------------------------------------------------------------------------------
# Differentiable photometric energy (forward / adjoint) and the inverse-depth refinement
# ------------------------------------------------------------------------------------------
def _ptr(a):
    return None if a is None else a.ctypes.data


def energy_points(key_image, key_idepth, key_var, intr, w, h, level=0, params=None):
    """(pixel index, initial inverse depth) of every energy point of a keyframe level."""
    p = params or default_params()
    f = lambda a: np.ascontiguousarray(a, np.float32)
    npx = (w >> level) * (h >> level)
    pix = np.zeros(npx, np.int32)
    rho0 = np.zeros(npx, np.float32)
    n = lib().lsdo_energy_points(f(key_image), f(key_idepth), f(key_var), w, h, C.byref(_intr(intr)), C.byref(p),
                                 level, pix.ctypes.data, rho0.ctypes.data)
    return pix[:n].copy(), rho0[:n].copy()


def energy(key_image, key_idepth, key_var, frame_image, intr, w, h, ref_to_frame, level=0, dof=6, rho=None,
           sigma2=None, fixed_active=None, grad=True, params=None, double=False):
    """E, dE/dxi (dof), dE/drho (per point), per-point energy terms, participation, broken count."""
    p = params or default_params()
    f = lambda a: np.ascontiguousarray(a, np.float32)
    n = len(energy_points(key_image, key_idepth, key_var, intr, w, h, level, p)[0])
    rho = None if rho is None else f(rho)
    sigma2 = None if sigma2 is None else f(sigma2)
    fixed_active = None if fixed_active is None else np.ascontiguousarray(fixed_active, np.uint8)
    gxi = np.zeros(7) if grad else None
    grho = np.zeros(n) if grad else None
    ept = np.zeros(n)
    act = np.zeros(n, np.uint8)
    E = np.zeros(1)
    na, nb = C.c_int(), C.c_int()
    rc = lib().lsdo_energy(int(double), f(key_image), f(key_idepth), f(key_var), f(frame_image), w, h,
                           C.byref(_intr(intr)), C.byref(p), level,
                           np.ascontiguousarray(ref_to_frame, np.float64).ravel(), dof, _ptr(rho), _ptr(sigma2),
                           _ptr(fixed_active), E.ctypes.data, _ptr(gxi), _ptr(grho), ept.ctypes.data, act.ctypes.data,
                           C.byref(na), C.byref(nb))
    assert rc == 0
    return dict(E=float(E[0]), gxi=None if gxi is None else gxi[:dof], grho=grho, e_point=ept, active=act,
                n_active=na.value, broken=nb.value)


def energy_refine(key_image, key_idepth, key_var, frame_images, ref_to_frames, intr, w, h, level=0, steps=50,
                  rho=None, sigma2=None, params=None, double=False, threads=None, fast=False):
    """Per-point inverse-depth refinement over the frames; returns (rho, E_before, E_after, refined)."""
    p = params or default_params()
    f = lambda a: np.ascontiguousarray(a, np.float32)
    if rho is None:
        rho = energy_points(key_image, key_idepth, key_var, intr, w, h, level, p)[1]
    rho = f(rho).copy()
    imgs = f(np.stack(frame_images))
    poses = np.ascontiguousarray(np.stack([np.asarray(T_, np.float64).reshape(3, 4) for T_ in ref_to_frames]))
    sigma2 = None if sigma2 is None else f(sigma2)
    e0, e1, cnt = C.c_double(), C.c_double(), C.c_long()
    rc = (fast_lib() if fast else lib()).lsdo_energy_refine(int(double), f(key_image), f(key_idepth), f(key_var), len(frame_images), imgs, w, h,
                                  C.byref(_intr(intr)), C.byref(p), level, poses.ravel(), steps, _ptr(sigma2), rho,
                                  C.byref(e0), C.byref(e1), C.byref(cnt), threads or hardware_threads())
    assert rc == 0
    return rho, e0.value, e1.value, cnt.value


# ------------------------------------------------------------------------------------------
# Keyframe point cloud (Keyframe::computeVbo)
# ------------------------------------------------------------------------------------------
POINT_DENSE = np.dtype([("idepth", "<f4"), ("idepth_var", "<f4"), ("color", "u1", (4,))])
CLOUD_VERTEX = np.dtype([("point", "<f4", (3,)), ("color", "u1", (4,))])


_ref_lib = None


def ref_lib():
    """The reference's own Keyframe::computeVbo loop compiled from its source (oracle/_ref, built by
    oracle/ref_build.py), or None where neither the reference tree nor its generated source is
    present."""
    global _ref_lib
    if _ref_lib is None:
        sys.path.insert(0, HERE)
        import ref_build as _rb  # oracle/ref_build.py
        path = _rb.build()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_compute_vbo.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.c_void_p, C.c_void_p]
        L.ref_compute_vbo.restype = C.c_int
        a, b = C.c_int(), C.c_int()
        L.ref_sizes(C.byref(a), C.byref(b))
        assert (a.value, b.value) == (POINT_DENSE.itemsize, CLOUD_VERTEX.itemsize)
        _ref_lib = L
    return _ref_lib


def ref_compute_vbo(points, w, h, fx, fy, cx, cy, scale=1.0):
    """Vertices computeVbo (the reference's code, its constants) keeps for a w x h InputPointDense
    array; None without oracle/_ref."""
    L = ref_lib()
    if L is None:
        return None
    pts = np.ascontiguousarray(points, POINT_DENSE).reshape(-1)
    assert pts.size == w * h
    out = np.zeros(w * h, CLOUD_VERTEX)
    n = L.ref_compute_vbo(w, h, fx, fy, cx, cy, scale, pts.ctypes.data, out.ctypes.data)
    return out[:n].copy()


def cloud_build(points, w, h, fx, fy, cx, cy, scale=1.0, scaled_th=1e-3, abs_th=1e-1, min_near_support=9):
    """Vertices (structured array) of a w x h InputPointDense array (structured, POINT_DENSE)."""
    pts = np.ascontiguousarray(points, POINT_DENSE).reshape(-1)
    assert pts.size == w * h
    out = np.zeros(w * h, CLOUD_VERTEX)
    p = T.CloudParams(scaled_th, abs_th, min_near_support, 0)
    n = lib().lsdo_cloud_build(w, h, fx, fy, cx, cy, scale, C.addressof(p), pts.ctypes.data, out.ctypes.data)
    return out[:n].copy()


# ------------------------------------------------------------------------------------------
# Input step: undistortion
# ------------------------------------------------------------------------------------------
def undistort_map(calib, out_w, out_h, K):
    """(out_h, out_w, 2) float32 source positions of the output pixels."""
    m = np.zeros((out_h, out_w, 2), np.float32)
    lib().lsdo_undistort_map(C.byref(calib), out_w, out_h, C.byref(_intr(K)), m.reshape(-1))
    return m


def undistort(raw, map_):
    raw = np.ascontiguousarray(raw, np.uint8)
    h, w = raw.shape
    out = np.zeros(map_.shape[:2], np.uint8)
    m = np.ascontiguousarray(map_, np.float32)
    lib().lsdo_undistort(raw.ctypes.data, w, h, m.reshape(-1), out.size, out.ctypes.data)
    return out
