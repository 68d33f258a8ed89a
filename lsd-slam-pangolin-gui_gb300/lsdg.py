"""Python view of the C-ABI (include/lsdg.h) through ctypes.

The classes mirror the upstream objects the reference's threads use:
``Frame`` (Frame: pyramid + optional keyframe depth), ``SE3Tracker.trackFrame``,
``Batch`` (many trackFrame calls in one persistent launch) and ``DepthMap``
(updateKeyframe / createKeyFrame / regularize).  Every call goes to liblsdg.so, whose kernels run
on the GPU; there is no CPU fallback and importing fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import lsdg_types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblsdg.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "lsdg.h")

_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_vp = C.c_void_p


class LsdgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{T.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _sig(L, name, restype, argtypes):
    f = getattr(L, name)
    f.restype = restype
    f.argtypes = argtypes


def lib():
    """Load liblsdg.so (built by build_lib.py).  Raises if it is absent: no fallback exists."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"liblsdg.so not built ({LIB_PATH}); run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    st = C.c_int
    _sig(L, "lsdg_abi_version", C.c_int32, [])
    _sig(L, "lsdg_default_params", None, [C.POINTER(T.Params)])
    _sig(L, "lsdg_create", st, [C.POINTER(_vp), C.POINTER(T.Params), C.c_int])
    _sig(L, "lsdg_destroy", st, [_vp])
    _sig(L, "lsdg_set_params", st, [_vp, C.POINTER(T.Params)])
    _sig(L, "lsdg_last_error", C.c_char_p, [_vp])
    _sig(L, "lsdg_stream", _vp, [_vp])
    _sig(L, "lsdg_sync", st, [_vp])
    _sig(L, "lsdg_launch_count", C.c_int64, [_vp])
    _sig(L, "lsdg_frame_create", st, [_vp, C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.POINTER(_vp)])
    _sig(L, "lsdg_frame_destroy", st, [_vp, _vp])
    _sig(L, "lsdg_frame_upload", st, [_vp, _vp, _f32p])
    _sig(L, "lsdg_frame_upload_u8", st, [_vp, _vp, _u8p])
    _sig(L, "lsdg_frame_set_depth", st, [_vp, _vp, _f32p, _f32p])
    _sig(L, "lsdg_frame_get_level", st, [_vp, _vp, C.c_int, _f32p])
    _sig(L, "lsdg_frame_get_depth", st, [_vp, _vp, C.c_int, _f32p, _f32p])
    _sig(L, "lsdg_frame_get_points", st, [_vp, _vp, C.c_int, _f32p, _f32p, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "lsdg_se3_normal_equations", st, [_vp, _vp, _vp, C.c_int, _f64p, _f64p])
    _sig(L, "lsdg_track_se3", st, [_vp, _vp, _vp, _f64p, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_sim3_normal_equations", st, [_vp, _vp, _vp, C.c_int, _f64p, _f64p])
    _sig(L, "lsdg_track_sim3", st, [_vp, _vp, _vp, _f64p, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_batch_create_sim3", st, [_vp, C.c_int, _i32p, _i32p, C.POINTER(T.Intrinsics), C.POINTER(_vp)])
    _sig(L, "lsdg_batch_load_sim3", st, [_vp, _vp] + [_vp] * 6 + [_f64p])
    _sig(L, "lsdg_batch_track_sim3", st, [_vp, _vp] + [_vp] * 6 + [_f64p, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_batch_create", st, [_vp, C.c_int, _i32p, _i32p, C.POINTER(T.Intrinsics), C.POINTER(_vp)])
    _sig(L, "lsdg_batch_destroy", st, [_vp, _vp])
    _sig(L, "lsdg_batch_load", st, [_vp, _vp, _vp, _vp, _vp, _vp, _f64p])
    _sig(L, "lsdg_batch_run", st, [_vp, _vp])
    _sig(L, "lsdg_batch_read", st, [_vp, _vp, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_batch_track_se3", st, [_vp, _vp, _vp, _vp, _vp, _vp, _f64p, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_batch_submit_se3", st, [_vp, _vp, _vp, _vp, _vp, _vp, _f64p])
    _sig(L, "lsdg_batch_submit_se3_u8", st, [_vp, _vp, _vp, _vp, _vp, _vp, _f64p])
    _sig(L, "lsdg_batch_submit_sim3", st, [_vp, _vp] + [_vp] * 6 + [_f64p])
    _sig(L, "lsdg_batch_load_frames", st, [_vp, _vp, _vp, _vp, _f64p])
    _sig(L, "lsdg_batch_collect", st, [_vp, _vp, _f64p, C.POINTER(T.TrackStats)])
    _sig(L, "lsdg_batch_timing", st, [_vp, _vp, C.POINTER(C.c_float), C.POINTER(C.c_float)])
    _sig(L, "lsdg_batch_shape", st, [_vp, _vp] + [C.POINTER(C.c_int)] * 5)
    _sig(L, "lsdg_batch_split", st, [_vp, _vp] + [C.POINTER(C.c_int)] * 4)
    _sig(L, "lsdg_batch_test_withhold", st, [_vp, _vp, C.c_int])
    _sig(L, "lsdg_batch_get_points", st, [_vp, _vp, C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "lsdg_batch_work", st, [_vp, _vp, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double)])
    _sig(L, "lsdg_depth_create", st, [_vp, C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.POINTER(_vp)])
    _sig(L, "lsdg_depth_destroy", st, [_vp, _vp])
    _sig(L, "lsdg_depth_set_keyframe", st, [_vp, _vp, _f32p, _f32p, _f32p])
    _sig(L, "lsdg_depth_load_refs", st, [_vp, _vp, C.c_int, _f32p])
    _sig(L, "lsdg_depth_update_loaded", st, [_vp, _vp, C.c_int, _f64p, C.c_int])
    _sig(L, "lsdg_depth_update", st, [_vp, _vp, C.c_int, _f32p, _f64p, C.c_int])
    _sig(L, "lsdg_depth_update_u8", st, [_vp, _vp, C.c_int, _vp, _f64p, C.c_int])
    _sig(L, "lsdg_depth_regularize", st, [_vp, _vp])
    _sig(L, "lsdg_depth_create_keyframe", st, [_vp, _vp, _f32p, _f64p, C.c_int])
    _sig(L, "lsdg_depth_get", st, [_vp, _vp] + [C.c_void_p] * 6)
    _sig(L, "lsdg_energy_create", st, [_vp, _vp, C.c_int, C.POINTER(_vp)])
    _sig(L, "lsdg_energy_destroy", st, [_vp, _vp])
    _sig(L, "lsdg_energy_size", st, [_vp, _vp, C.POINTER(C.c_int)])
    _sig(L, "lsdg_energy_pixels", st, [_vp, _vp, _i32p])
    _sig(L, "lsdg_energy_set_idepth", st, [_vp, _vp, _vp])
    _sig(L, "lsdg_energy_get_idepth", st, [_vp, _vp, _f32p])
    _sig(L, "lsdg_energy_set_sigma2", st, [_vp, _vp, _vp])
    _sig(L, "lsdg_energy_forward", st, [_vp, _vp, _vp, _f64p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)])
    _sig(L, "lsdg_energy_backward", st, [_vp, _vp, C.c_double, _f64p, _vp])
    _sig(L, "lsdg_energy_refine", st, [_vp, _vp, C.c_int, _vp, _f64p, C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int)])
    _sig(L, "lsdg_energy_timing", st, [_vp, _vp] + [C.POINTER(C.c_float)] * 3)
    _sig(L, "lsdg_cloud_default_params", None, [C.POINTER(T.CloudParams)])
    _sig(L, "lsdg_depth_export_points", st, [_vp, _vp, _vp])
    _sig(L, "lsdg_cloud_build", st, [_vp, C.c_int, C.c_int] + [C.c_float] * 5 + [C.POINTER(T.CloudParams), _vp, _vp,
                                                                                 C.POINTER(C.c_int)])
    _sig(L, "lsdg_cloud_from_depthmap", st, [_vp, _vp, C.c_float, C.POINTER(T.CloudParams), _vp, C.POINTER(C.c_int)])
    _sig(L, "lsdg_calibration_load_xml", st, [C.c_char_p, C.POINTER(T.Calibration)])
    _sig(L, "lsdg_undistorter_create", st, [_vp, C.POINTER(T.Calibration), C.c_int, C.c_int, C.POINTER(T.Intrinsics),
                                            C.POINTER(_vp)])
    _sig(L, "lsdg_undistorter_destroy", st, [_vp, _vp])
    _sig(L, "lsdg_undistorter_camera", st, [_vp, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(T.Intrinsics)])
    _sig(L, "lsdg_frame_upload_distorted_u8", st, [_vp, _vp, _vp, _u8p])
    _sig(L, "lsdg_undistorter_last_image", st, [_vp, _vp, _u8p])
    _sig(L, "lsdg_sim3_to_sophus7", None, [_f64p, _f32p])
    _sig(L, "lsdg_sophus7_to_sim3", None, [_f32p, _f64p])
    _sig(L, "lsdg_format_pose_row", C.c_int, [C.c_int, _f64p, _f64p, C.c_char_p, C.c_int])
    _sig(L, "lsdg_tune_info", st, [_vp, C.c_int, C.c_char_p, C.c_int] + [C.POINTER(C.c_int)] * 4 + [C.POINTER(C.c_float)])
    _sig(L, "lsdg_slam_default_params", None, [C.POINTER(T.SlamParams)])
    _sig(L, "lsdg_slam_create", st, [C.POINTER(T.Params), C.POINTER(T.SlamParams), C.c_int, C.c_int, C.c_int,
                                     C.POINTER(T.Intrinsics), C.POINTER(_vp)])
    _sig(L, "lsdg_slam_destroy", st, [_vp])
    _sig(L, "lsdg_slam_last_error", C.c_char_p, [_vp])
    _sig(L, "lsdg_slam_bootstrap", st, [_vp, C.c_int, _u8p, _f32p, _f32p])
    _sig(L, "lsdg_slam_next_image", st, [_vp, C.c_int, _u8p])
    _sig(L, "lsdg_slam_finalize", st, [_vp])
    _sig(L, "lsdg_slam_get_stats", st, [_vp, C.POINTER(T.SlamStats)])
    _sig(L, "lsdg_slam_get_poses", st, [_vp, _vp, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "lsdg_slam_keyframe_graph", st, [_vp, _vp, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "lsdg_slam_write_pose_file", st, [_vp, C.c_char_p])
    _sig(L, "lsdg_slam_keyframe_depth", st, [_vp, C.c_int, C.POINTER(C.c_int), _f32p, _f32p])
    _sig(L, "lsdg_posegraph_create", st, [C.POINTER(_vp)])
    _sig(L, "lsdg_posegraph_destroy", st, [_vp])
    _sig(L, "lsdg_posegraph_add_node", C.c_int, [_vp, _f64p])
    _sig(L, "lsdg_posegraph_add_edge", st, [_vp, C.c_int, C.c_int, _f64p, _f64p])
    _sig(L, "lsdg_posegraph_optimize", st, [_vp, C.c_int, C.POINTER(C.c_double)])
    _sig(L, "lsdg_posegraph_get_pose", st, [_vp, C.c_int, _f64p])
    _sig(L, "lsdg_sim3_exp13", None, [_f64p, _f64p])
    _sig(L, "lsdg_sim3_log13", None, [_f64p, _f64p])
    _sig(L, "lsdg_measure_l2_read", st, [_vp, C.c_long, C.c_int, C.POINTER(C.c_double)])
    _lib = L
    return L


def default_params() -> T.Params:
    p = T.Params()
    lib().lsdg_default_params(C.byref(p))
    return p


def intrinsics(intr) -> T.Intrinsics:
    if isinstance(intr, T.Intrinsics):
        return intr
    fx, fy, cx, cy = intr.as_tuple() if hasattr(intr, "as_tuple") else intr
    return T.Intrinsics(fx, fy, cx, cy)


def _pose12(p) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(p, np.float64).reshape(-1))
    assert a.size == 12
    return a


class Context:
    """One CUDA stream on one device (upstream: one of SlamSystem's threads)."""

    def __init__(self, params: T.Params = None, device: int = 0):
        self._h = _vp()
        self.params = (params or default_params()).copy()
        rc = lib().lsdg_create(C.byref(self._h), C.byref(self.params), device)
        if rc != T.OK:
            raise LsdgError(rc, "lsdg_create failed")

    @property
    def handle(self):
        return self._h

    def check(self, rc: int, allow=(T.OK,)):
        if rc not in allow:
            raise LsdgError(rc, (lib().lsdg_last_error(self._h) or b"").decode())
        return rc

    def set_params(self, p: T.Params):
        self.check(lib().lsdg_set_params(self._h, C.byref(p)))
        self.params = p.copy()

    def stream_ptr(self) -> int:
        return lib().lsdg_stream(self._h) or 0

    def sync(self):
        self.check(lib().lsdg_sync(self._h))

    def launch_count(self) -> int:
        return int(lib().lsdg_launch_count(self._h))

    def tune_table(self):
        out, i = [], 0
        buf = C.create_string_buffer(256)
        while True:
            t, mb, c, m, ms = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_float()
            rc = lib().lsdg_tune_info(self._h, i, buf, 256, C.byref(t), C.byref(mb), C.byref(c), C.byref(m), C.byref(ms))
            if rc != T.OK:
                return out
            out.append({"key": buf.value.decode(), "threads": t.value, "minblocks": mb.value, "cluster": c.value,
                        "clusters": m.value, "ms": ms.value})
            i += 1

    def close(self):
        if self._h:
            lib().lsdg_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Frame:
    """Upstream Frame: intensity + gradient pyramid; a keyframe also carries inverse depth."""

    def __init__(self, ctx: Context, width: int, height: int, intr):
        self.ctx, self.w, self.h = ctx, width, height
        self.levels = ctx.params.levels
        self._h = _vp()
        self._k = intrinsics(intr)
        ctx.check(lib().lsdg_frame_create(ctx.handle, width, height, C.byref(self._k), C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def upload(self, image: np.ndarray):
        if image.dtype == np.uint8:
            self.ctx.check(lib().lsdg_frame_upload_u8(self.ctx.handle, self._h, np.ascontiguousarray(image)))
        else:
            self.ctx.check(lib().lsdg_frame_upload(self.ctx.handle, self._h, np.ascontiguousarray(image, np.float32)))
        return self

    def set_depth(self, idepth: np.ndarray, idepth_var: np.ndarray):
        self.ctx.check(lib().lsdg_frame_set_depth(self.ctx.handle, self._h, np.ascontiguousarray(idepth, np.float32),
                                                  np.ascontiguousarray(idepth_var, np.float32)))
        return self

    def level(self, l: int) -> np.ndarray:
        out = np.zeros(((self.h >> l), (self.w >> l), 4), np.float32)
        self.ctx.check(lib().lsdg_frame_get_level(self.ctx.handle, self._h, l, out.reshape(-1)))
        return out

    def depth(self, l: int):
        d = np.zeros(((self.h >> l), (self.w >> l)), np.float32)
        v = np.zeros_like(d)
        self.ctx.check(lib().lsdg_frame_get_depth(self.ctx.handle, self._h, l, d.reshape(-1), v.reshape(-1)))
        return d, v

    def points(self, l: int):
        cap = (self.w >> l) * (self.h >> l)
        xyzi = np.zeros(4 * cap, np.float32)
        var = np.zeros(cap, np.float32)
        n = C.c_int()
        self.ctx.check(lib().lsdg_frame_get_points(self.ctx.handle, self._h, l, xyzi, var, cap, C.byref(n)))
        return xyzi[:4 * n.value].reshape(-1, 4), var[:n.value]

    def close(self):
        if self._h and self.ctx.handle:
            lib().lsdg_frame_destroy(self.ctx.handle, self._h)
        self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def se3_normal_equations(ctx: Context, reference: Frame, frame: Frame, level: int, ref_to_frame) -> np.ndarray:
    """calculateWarpUpdate at a fixed pose: the LSDG_NE_SIZE record (see include/lsdg.h)."""
    out = np.zeros(T.NE_SIZE, np.float64)
    ctx.check(lib().lsdg_se3_normal_equations(ctx.handle, reference.handle, frame.handle, level, _pose12(ref_to_frame), out))
    return out


def _pose13(p) -> np.ndarray:
    """A Sim3 pose as 13 doubles {R (row-major), t, s}; accepts (R|t 3x4, s) tuples or 13 values."""
    if isinstance(p, tuple):
        M = np.asarray(p[0], np.float64).reshape(3, 4)
        a = np.concatenate([M[:, :3].ravel(), M[:, 3], [float(p[1])]])
    else:
        a = np.asarray(p, np.float64).reshape(-1)
    a = np.ascontiguousarray(a)
    assert a.size == 13
    return a


def unpack13(p):
    """13 doubles {R (row-major), t, s} -> ([R | t] 3x4, s)."""
    p = np.asarray(p, np.float64).reshape(-1)
    M = np.zeros((3, 4))
    M[:, :3] = p[:9].reshape(3, 3)
    M[:, 3] = p[9:12]
    return M, float(p[12])


def sim3_normal_equations(ctx: Context, reference: Frame, frame: Frame, level: int, ref_to_frame) -> np.ndarray:
    """One Sim3 residual pass at a fixed pose: the LSDG_NE_SIZE_SIM3 record (see include/lsdg.h)."""
    out = np.zeros(T.NE_SIZE_SIM3, np.float64)
    ctx.check(lib().lsdg_sim3_normal_equations(ctx.handle, reference.handle, frame.handle, level,
                                               _pose13(ref_to_frame), out))
    return out


class SE3Tracker:
    """Upstream SE3Tracker: trackFrame(reference, frame, frameToReference_initialEstimate)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.last_stats = T.TrackStats()

    def trackFrame(self, reference: Frame, frame: Frame, frame_to_ref_init=None):
        init = _pose12(np.eye(3, 4) if frame_to_ref_init is None else frame_to_ref_init)
        out = np.zeros(12, np.float64)
        st = T.TrackStats()
        self.ctx.check(lib().lsdg_track_se3(self.ctx.handle, reference.handle, frame.handle, init, out, C.byref(st)),
                       allow=(T.OK, T.TRACKING_LOST))
        self.last_stats = st
        return out.reshape(3, 4), st


class Sim3Tracker:
    """Upstream Sim3Tracker: trackFrameSim3(reference, frame, frameToReference_initialEstimate).

    Poses are (R|t 3x4, scale) tuples; both keyframes need depth (Frame.set_depth)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.last_stats = T.TrackStats()

    def trackFrameSim3(self, reference: Frame, frame: Frame, frame_to_ref_init=None):
        init = _pose13((np.eye(3, 4), 1.0) if frame_to_ref_init is None else frame_to_ref_init)
        out = np.zeros(13, np.float64)
        st = T.TrackStats()
        self.ctx.check(lib().lsdg_track_sim3(self.ctx.handle, reference.handle, frame.handle, init, out, C.byref(st)),
                       allow=(T.OK, T.TRACKING_LOST))
        self.last_stats = st
        return unpack13(out), st


class Batch:
    """Many independent trackFrame calls of mixed size in one persistent launch (graph-captured).

    sim3=True makes a batch of Sim3 constraint trackings (both keyframes with depth, 13-double poses)."""

    def __init__(self, ctx: Context, widths, heights, intrs, sim3: bool = False):
        self.ctx = ctx
        self.n = len(widths)
        self.sim3 = sim3
        self.widths = np.ascontiguousarray(widths, np.int32)
        self.heights = np.ascontiguousarray(heights, np.int32)
        self._k = (T.Intrinsics * self.n)(*[intrinsics(k) for k in intrs])
        self._h = _vp()
        create = lib().lsdg_batch_create_sim3 if sim3 else lib().lsdg_batch_create
        ctx.check(create(ctx.handle, self.n, self.widths, self.heights, self._k, C.byref(self._h)))
        self.npix = int(np.sum(self.widths.astype(np.int64) * self.heights))
        self.plen = 13 if sim3 else 12

    @staticmethod
    def _ptr(a: np.ndarray):
        assert a.flags["C_CONTIGUOUS"] and a.dtype == np.float32
        return a.ctypes.data

    def load(self, ref_images, ref_idepth, ref_var, new_images, init):
        """Host arrays (ideally pinned) holding the pairs' planes back to back; init (n,3,4)."""
        for a in (ref_images, ref_idepth, ref_var, new_images):
            assert a.size == self.npix, (a.size, self.npix)
        self._keep = (ref_images, ref_idepth, ref_var, new_images)
        self.ctx.check(lib().lsdg_batch_load(self.ctx.handle, self._h, self._ptr(ref_images), self._ptr(ref_idepth),
                                             self._ptr(ref_var), self._ptr(new_images),
                                             np.ascontiguousarray(init, np.float64).reshape(-1)))

    def load_sim3(self, ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var, init):
        """Sim3 batch: init is (n, 13) {R, t, s} per pair."""
        arrs = (ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var)
        for a in arrs:
            assert a.size == self.npix, (a.size, self.npix)
        self._keep = arrs
        self.ctx.check(lib().lsdg_batch_load_sim3(self.ctx.handle, self._h, *[self._ptr(a) for a in arrs],
                                                  np.ascontiguousarray(init, np.float64).reshape(-1)))

    def submit(self, ref_images, ref_idepth, ref_var, new_images, init):
        """Pipelined step (lsdg_batch_submit_se3): returns at once; collect() gives its results.
        The arrays must stay untouched (and should be pinned) until then."""
        arrs = (ref_images, ref_idepth, ref_var, new_images)
        for a in arrs:
            assert a.size == self.npix, (a.size, self.npix)
        self._pending = getattr(self, "_pending", []) + [arrs]
        self.ctx.check(lib().lsdg_batch_submit_se3(self.ctx.handle, self._h, *[self._ptr(a) for a in arrs],
                                                   np.ascontiguousarray(init, np.float64).reshape(-1)))

    def submit_u8(self, ref_images, ref_idepth, ref_var, new_images, init):
        """submit() with 8-bit images (lsdg_batch_submit_se3_u8): the bytes cross the bus and are
        widened on the device; results equal submit() with the same images as floats."""
        for a in (ref_images, new_images):
            assert a.dtype == np.uint8 and a.flags["C_CONTIGUOUS"] and a.size == self.npix, (a.dtype, a.size, self.npix)
        for a in (ref_idepth, ref_var):
            assert a.size == self.npix, (a.size, self.npix)
        arrs = (ref_images, ref_idepth, ref_var, new_images)
        self._pending = getattr(self, "_pending", []) + [arrs]
        self.ctx.check(lib().lsdg_batch_submit_se3_u8(self.ctx.handle, self._h, ref_images.ctypes.data,
                                                      self._ptr(ref_idepth), self._ptr(ref_var), new_images.ctypes.data,
                                                      np.ascontiguousarray(init, np.float64).reshape(-1)))

    def submit_sim3(self, ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var, init):
        arrs = (ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var)
        for a in arrs:
            assert a.size == self.npix, (a.size, self.npix)
        self._pending = getattr(self, "_pending", []) + [arrs]
        self.ctx.check(lib().lsdg_batch_submit_sim3(self.ctx.handle, self._h, *[self._ptr(a) for a in arrs],
                                                    np.ascontiguousarray(init, np.float64).reshape(-1)))

    def collect(self):
        """Results of the oldest submitted step."""
        out = np.zeros(self.plen * self.n, np.float64)
        stats = (T.TrackStats * self.n)()
        self.ctx.check(lib().lsdg_batch_collect(self.ctx.handle, self._h, out, stats))
        self._pending = self._pending[1:]
        return (out.reshape(self.n, 13) if self.sim3 else out.reshape(self.n, 3, 4)), stats

    def load_frames(self, refs, frames, init):
        """Fill the batch from resident Frames (device-to-device); init (n, 12) or (n, 13)."""
        assert len(refs) == len(frames) == self.n
        ra = (_vp * self.n)(*[f.handle for f in refs])
        fa = (_vp * self.n)(*[f.handle for f in frames])
        self.ctx.check(lib().lsdg_batch_load_frames(self.ctx.handle, self._h, ra, fa,
                                                    np.ascontiguousarray(init, np.float64).reshape(-1)))

    def run(self):
        self.ctx.check(lib().lsdg_batch_run(self.ctx.handle, self._h))

    def read(self):
        out = np.zeros(self.plen * self.n, np.float64)
        stats = (T.TrackStats * self.n)()
        self.ctx.check(lib().lsdg_batch_read(self.ctx.handle, self._h, out, stats))
        if self.sim3:
            return out.reshape(self.n, 13), stats
        return out.reshape(self.n, 3, 4), stats

    def track(self, ref_images, ref_idepth, ref_var, new_images, init):
        out = np.zeros(12 * self.n, np.float64)
        stats = (T.TrackStats * self.n)()
        self.ctx.check(lib().lsdg_batch_track_se3(self.ctx.handle, self._h, self._ptr(ref_images), self._ptr(ref_idepth),
                                                  self._ptr(ref_var), self._ptr(new_images),
                                                  np.ascontiguousarray(init, np.float64).reshape(-1), out, stats))
        return out.reshape(self.n, 3, 4), stats

    def timing(self):
        a, b = C.c_float(), C.c_float()
        self.ctx.check(lib().lsdg_batch_timing(self.ctx.handle, self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def shape(self):
        t, mb, c, n, k = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.ctx.check(lib().lsdg_batch_shape(self.ctx.handle, self._h, C.byref(t), C.byref(mb), C.byref(c), C.byref(n),
                                              C.byref(k)))
        sp, ct, cm, cc = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.ctx.check(lib().lsdg_batch_split(self.ctx.handle, self._h, C.byref(sp), C.byref(ct), C.byref(cm),
                                              C.byref(cc)))
        out = {"threads": t.value, "minblocks": mb.value, "cluster": c.value, "clusters": n.value,
               "launches_per_run": k.value}
        if sp.value >= 0:
            out["coarse_phase"] = {"levels_from": sp.value, "threads": ct.value, "minblocks": cm.value,
                                   "cluster": cc.value}
        return out

    def test_withhold(self, frame: int):
        """Test hook of the build's bounded wait (lsdg_batch_test_withhold; -1 turns it off)."""
        self.ctx.check(lib().lsdg_batch_test_withhold(self.ctx.handle, self._h, frame))

    def points(self, pair: int, l: int):
        """Reference points the last step built for pair `pair`'s keyframe at level l: (n, 4), (n,)."""
        cap = (int(self.widths[pair]) >> l) * (int(self.heights[pair]) >> l)
        xyzi = np.zeros(4 * cap, np.float32)
        var = np.zeros(cap, np.float32)
        n = C.c_int()
        self.ctx.check(lib().lsdg_batch_get_points(self.ctx.handle, self._h, pair, l, xyzi, var, cap, C.byref(n)))
        return xyzi[:4 * n.value].reshape(-1, 4), var[:n.value]

    def work(self):
        p, b, u = C.c_int64(), C.c_double(), C.c_double()
        self.ctx.check(lib().lsdg_batch_work(self.ctx.handle, self._h, C.byref(p), C.byref(b), C.byref(u)))
        return p.value, b.value, u.value

    def close(self):
        if self._h and self.ctx.handle:
            lib().lsdg_batch_destroy(self.ctx.handle, self._h)
        self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DepthMap:
    """Upstream DepthMap: semi-dense inverse-depth hypotheses of one keyframe on the GPU."""

    PLANES = ("idepth", "var", "idepth_smoothed", "var_smoothed", "validity", "blacklist")

    def __init__(self, ctx: Context, width: int, height: int, intr):
        self.ctx, self.w, self.h = ctx, width, height
        self._k = intrinsics(intr)
        self._h = _vp()
        ctx.check(lib().lsdg_depth_create(ctx.handle, width, height, C.byref(self._k), C.byref(self._h)))

    def set_keyframe(self, image, idepth, idepth_var):
        self.ctx.check(lib().lsdg_depth_set_keyframe(self.ctx.handle, self._h, np.ascontiguousarray(image, np.float32),
                                                     np.ascontiguousarray(idepth, np.float32),
                                                     np.ascontiguousarray(idepth_var, np.float32)))
        return self

    @staticmethod
    def _refs(ref_images, key_to_ref):
        imgs = np.ascontiguousarray(np.concatenate([np.asarray(r, np.float32).ravel() for r in ref_images]), np.float32)
        poses = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1) for p in key_to_ref]))
        return imgs, poses

    def updateKeyframe(self, ref_images, key_to_ref, regularize=True):
        imgs, poses = self._refs(ref_images, key_to_ref)
        self.ctx.check(lib().lsdg_depth_update(self.ctx.handle, self._h, len(ref_images), imgs, poses, int(regularize)))

    def updateKeyframe_u8(self, ref_images_u8, key_to_ref, regularize=True):
        """8-bit reference frames: one (n, h, w) uint8 array (pinned for speed) or a list of (h, w)."""
        a = ref_images_u8 if isinstance(ref_images_u8, np.ndarray) else np.stack(ref_images_u8)
        assert a.dtype == np.uint8 and a.flags["C_CONTIGUOUS"] and a.size % (self.w * self.h) == 0
        n = a.size // (self.w * self.h)
        poses = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1) for p in key_to_ref]))
        self.ctx.check(lib().lsdg_depth_update_u8(self.ctx.handle, self._h, n, a.ctypes.data, poses, int(regularize)))

    def load_refs(self, ref_images):
        imgs = np.ascontiguousarray(np.concatenate([np.asarray(r, np.float32).ravel() for r in ref_images]), np.float32)
        self._keep = imgs
        self.ctx.check(lib().lsdg_depth_load_refs(self.ctx.handle, self._h, len(ref_images), imgs))

    def update_loaded(self, key_to_ref, regularize=True):
        poses = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1) for p in key_to_ref]))
        self.ctx.check(lib().lsdg_depth_update_loaded(self.ctx.handle, self._h, len(key_to_ref), poses, int(regularize)))

    def regularize(self):
        self.ctx.check(lib().lsdg_depth_regularize(self.ctx.handle, self._h))

    def export_points(self):
        """publishKeyframe's InputPointDense array (h, w) of the current keyframe."""
        out = np.zeros(self.w * self.h, POINT_DENSE)
        self.ctx.check(lib().lsdg_depth_export_points(self.ctx.handle, self._h, out.ctypes.data))
        return out.reshape(self.h, self.w)

    def cloud_to_device(self, device_ptr: int, scale: float = 1.0, params=None) -> int:
        """Keyframe::computeVbo of the current keyframe into a device buffer (w * h vertices of
        16 bytes, 16-byte aligned); returns the vertex count."""
        n = C.c_int()
        self.ctx.check(lib().lsdg_cloud_from_depthmap(self.ctx.handle, self._h, scale,
                                                      None if params is None else C.byref(params),
                                                      C.c_void_p(device_ptr), C.byref(n)))
        return n.value

    def createKeyFrame(self, new_image, key_to_new, regularize=True):
        self.ctx.check(lib().lsdg_depth_create_keyframe(self.ctx.handle, self._h, np.ascontiguousarray(new_image, np.float32),
                                                        _pose12(key_to_new), int(regularize)))

    def get(self, planes=None, out=None):
        """The state planes (all by default); `out` may hold preallocated (e.g. pinned) arrays."""
        planes = self.PLANES if planes is None else planes
        out = {} if out is None else out
        for name in planes:
            if name not in out:
                dt = np.int32 if name in ("validity", "blacklist") else np.float32
                out[name] = np.zeros((self.h, self.w), dt)
        ptrs = [out[n].ctypes.data if n in planes else None for n in self.PLANES]
        self.ctx.check(lib().lsdg_depth_get(self.ctx.handle, self._h, *ptrs))
        return out

    def close(self):
        if self._h and self.ctx.handle:
            lib().lsdg_depth_destroy(self.ctx.handle, self._h)
        self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PhotometricEnergy:
    """The photometric energy of a keyframe level against a frame, as an autograd Function:
    forward(frame, ref_to_frame, dof) -> E saves the pose and the inverse depths' version;
    backward(grad_E) -> (dL/dxi, dL/drho) recomputes the residuals.  refine() runs the per-point
    inverse-depth refinement over several frames."""

    def __init__(self, ctx: Context, keyframe: Frame, level: int = 0):
        self.ctx = ctx
        self._h = _vp()
        ctx.check(lib().lsdg_energy_create(ctx.handle, keyframe.handle, level, C.byref(self._h)))
        n = C.c_int()
        ctx.check(lib().lsdg_energy_size(ctx.handle, self._h, C.byref(n)))
        self.n = n.value
        self.dof = 6

    def pixels(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.int32)
        self.ctx.check(lib().lsdg_energy_pixels(self.ctx.handle, self._h, out))
        return out[:self.n]

    def idepth(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.float32)
        self.ctx.check(lib().lsdg_energy_get_idepth(self.ctx.handle, self._h, out))
        return out[:self.n]

    def set_idepth(self, rho=None):
        a = None if rho is None else np.ascontiguousarray(rho, np.float32)
        if a is not None:
            assert a.size == self.n
        self.ctx.check(lib().lsdg_energy_set_idepth(self.ctx.handle, self._h, None if a is None else a.ctypes.data))

    def set_sigma2(self, sigma2=None):
        a = None if sigma2 is None else np.ascontiguousarray(sigma2, np.float32)
        if a is not None:
            assert a.size == self.n
        self.ctx.check(lib().lsdg_energy_set_sigma2(self.ctx.handle, self._h, None if a is None else a.ctypes.data))

    def forward(self, frame: Frame, ref_to_frame, dof: int = 6):
        E, na = C.c_double(), C.c_int()
        self.ctx.check(lib().lsdg_energy_forward(self.ctx.handle, self._h, frame.handle, _pose12(ref_to_frame), dof,
                                                 C.byref(E), C.byref(na)))
        self.dof = dof
        self.n_active = na.value
        return E.value

    def backward(self, grad_energy: float = 1.0, want_idepth: bool = True):
        gxi = np.zeros(7)
        grho = np.zeros(max(self.n, 1), np.float32) if want_idepth else None
        self.ctx.check(lib().lsdg_energy_backward(self.ctx.handle, self._h, float(grad_energy), gxi,
                                                  None if grho is None else grho.ctypes.data))
        return gxi[:self.dof], (None if grho is None else grho[:self.n])

    def refine(self, frames, ref_to_frames, steps: int = 50):
        arr = (_vp * len(frames))(*[f.handle for f in frames])
        poses = np.ascontiguousarray(np.stack([np.asarray(T_, np.float64).reshape(3, 4) for T_ in ref_to_frames]))
        e0, e1, nr = C.c_double(), C.c_double(), C.c_int()
        self.ctx.check(lib().lsdg_energy_refine(self.ctx.handle, self._h, len(frames), arr, poses.ravel(), steps,
                                                C.byref(e0), C.byref(e1), C.byref(nr)))
        return e0.value, e1.value, nr.value

    def timing(self):
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        self.ctx.check(lib().lsdg_energy_timing(self.ctx.handle, self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        if self._h and self.ctx.handle:
            lib().lsdg_energy_destroy(self.ctx.handle, self._h)
        self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sim3_to_sophus7(pose13) -> np.ndarray:
    """13-double {R, t, s} -> the 7 floats of Sophus::Sim3f::data() (quaternion x y z w with
    squared norm = scale, translation) that GraphFramePose carries."""
    out = np.zeros(7, np.float32)
    lib().lsdg_sim3_to_sophus7(_pose13(pose13), out)
    return out


def sophus7_to_sim3(p7) -> np.ndarray:
    out = np.zeros(13, np.float64)
    lib().lsdg_sophus7_to_sim3(np.ascontiguousarray(p7, np.float32), out)
    return out


def format_pose_row(frame_id: int, cam_to_world13, this_to_parent13) -> str:
    buf = C.create_string_buffer(256)
    n = lib().lsdg_format_pose_row(frame_id, _pose13(cam_to_world13), _pose13(this_to_parent13), buf, 256)
    assert n > 0
    return buf.value.decode()


def calibration_load_xml(path: str) -> T.Calibration:
    """Parse a calibration file (d2_camera.xml format) with the library's reader (host only)."""
    c = T.Calibration()
    rc = lib().lsdg_calibration_load_xml(path.encode(), C.byref(c))
    if rc != T.OK:
        raise LsdgError(rc, "cannot read calibration %s" % path)
    return c


class Undistorter:
    """The input thread's undistorter: raw 8-bit frames of the calibrated camera -> frames of the
    ideal pinhole output camera (camera())."""

    def __init__(self, ctx: Context, calib: T.Calibration, out_w: int = None, out_h: int = None, out_K=None):
        self.ctx = ctx
        self.calib = calib
        self._h = _vp()
        ow = calib.width if out_w is None else out_w
        oh = calib.height if out_h is None else out_h
        k = None if out_K is None else C.byref(intrinsics(out_K))
        ctx.check(lib().lsdg_undistorter_create(ctx.handle, C.byref(calib), ow, oh, k, C.byref(self._h)))

    def camera(self):
        w, h, k = C.c_int(), C.c_int(), T.Intrinsics()
        self.ctx.check(lib().lsdg_undistorter_camera(self.ctx.handle, self._h, C.byref(w), C.byref(h), C.byref(k)))
        return w.value, h.value, k

    def upload(self, frame: "Frame", raw: np.ndarray):
        raw = np.ascontiguousarray(raw, np.uint8)
        assert raw.shape == (self.calib.height, self.calib.width)
        self.ctx.check(lib().lsdg_frame_upload_distorted_u8(self.ctx.handle, self._h, frame.handle, raw.reshape(-1)))
        return frame

    def last_image(self):
        w, h, _ = self.camera()
        out = np.zeros(w * h, np.uint8)
        self.ctx.check(lib().lsdg_undistorter_last_image(self.ctx.handle, self._h, out))
        return out.reshape(h, w)

    def close(self):
        if self._h and self.ctx.handle:
            lib().lsdg_undistorter_destroy(self.ctx.handle, self._h)
        self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


POINT_DENSE = np.dtype([("idepth", "<f4"), ("idepth_var", "<f4"), ("color", "u1", (4,))])  # InputPointDense
CLOUD_VERTEX = np.dtype([("point", "<f4", (3,)), ("color", "u1", (4,))])                     # Keyframe::MyVertex


def cloud_default_params() -> T.CloudParams:
    p = T.CloudParams()
    lib().lsdg_cloud_default_params(C.byref(p))
    return p


def cloud_build(ctx: Context, points, w: int, h: int, fx, fy, cx, cy, scale: float = 1.0, params=None):
    """Keyframe::computeVbo on the GPU: vertices (structured CLOUD_VERTEX array) of a w x h
    InputPointDense array."""
    pts = np.ascontiguousarray(points, POINT_DENSE).reshape(-1)
    assert pts.size == w * h
    out = np.zeros(w * h, CLOUD_VERTEX)
    n = C.c_int()
    ctx.check(lib().lsdg_cloud_build(ctx.handle, w, h, fx, fy, cx, cy, scale,
                                     None if params is None else C.byref(params), pts.ctypes.data, out.ctypes.data,
                                     C.byref(n)))
    return out[:n.value].copy()


def measure_l2_read(ctx: "Context", bytes_: int = 32 << 20, reps: int = 50) -> float:
    """L2 read bandwidth (GB/s) of an L2-resident buffer on the context's GPU."""
    g = C.c_double()
    ctx.check(lib().lsdg_measure_l2_read(ctx.handle, bytes_, reps, C.byref(g)))
    return g.value


def slam_default_params() -> T.SlamParams:
    p = T.SlamParams()
    lib().lsdg_slam_default_params(C.byref(p))
    return p


class SlamSystem:
    """Upstream SlamSystem over the C-ABI (lsdg_slam_*): nextImage tracks and maps a frame on the
    caller's thread; keyframes' Sim3 constraint search and the pose graph run on the library's
    worker thread."""

    def __init__(self, w: int, h: int, intr, params: T.Params = None, slam_params: T.SlamParams = None,
                 device: int = 0):
        self.w, self.h = w, h
        self._h = _vp()
        p = params or default_params()
        sp = slam_params or slam_default_params()
        rc = lib().lsdg_slam_create(C.byref(p), C.byref(sp), device, w, h, C.byref(intrinsics(intr)), C.byref(self._h))
        if rc != T.OK:
            raise LsdgError(rc, "lsdg_slam_create")

    def _check(self, rc):
        if rc != T.OK:
            raise LsdgError(rc, lib().lsdg_slam_last_error(self._h).decode())

    def bootstrap(self, frame_id: int, image_u8, idepth, var):
        self._check(lib().lsdg_slam_bootstrap(self._h, frame_id, np.ascontiguousarray(image_u8, np.uint8),
                                              np.ascontiguousarray(idepth, np.float32),
                                              np.ascontiguousarray(var, np.float32)))

    def nextImage(self, frame_id: int, image_u8):
        self._check(lib().lsdg_slam_next_image(self._h, frame_id, np.ascontiguousarray(image_u8, np.uint8)))

    def finalize(self):
        self._check(lib().lsdg_slam_finalize(self._h))

    def stats(self) -> dict:
        st = T.SlamStats()
        self._check(lib().lsdg_slam_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in T.SlamStats._fields_ if k != "reserved"}

    def poses(self) -> np.ndarray:
        """(n, 13) camera-to-world Sim3 {R, t, s} of every frame."""
        n = C.c_int()
        self._check(lib().lsdg_slam_get_poses(self._h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 13))
        self._check(lib().lsdg_slam_get_poses(self._h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def keyframe_graph(self):
        n = C.c_int()
        self._check(lib().lsdg_slam_keyframe_graph(self._h, None, 0, C.byref(n)))
        arr = (T.GraphFramePose * n.value)()
        self._check(lib().lsdg_slam_keyframe_graph(self._h, C.cast(arr, _vp), n.value, C.byref(n)))
        return [(g.id, np.array(g.cam_to_world[:], np.float32)) for g in arr]

    def keyframe_depth(self, k: int):
        """(frame id, inverse depth [h, w], variance [h, w]) of keyframe k."""
        fid = C.c_int()
        d = np.zeros((self.h, self.w), np.float32)
        v = np.zeros((self.h, self.w), np.float32)
        self._check(lib().lsdg_slam_keyframe_depth(self._h, k, C.byref(fid), d, v))
        return fid.value, d, v

    def write_pose_file(self, path: str):
        self._check(lib().lsdg_slam_write_pose_file(self._h, path.encode()))

    def close(self):
        if self._h:
            lib().lsdg_slam_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NativePoseGraph:
    """The library's Sim3 pose graph (lsdg_posegraph_*), poses as 13-double {R, t, s}."""

    def __init__(self):
        self._h = _vp()
        rc = lib().lsdg_posegraph_create(C.byref(self._h))
        if rc != T.OK:
            raise LsdgError(rc, "lsdg_posegraph_create")

    def add_node(self, pose13) -> int:
        return lib().lsdg_posegraph_add_node(self._h, np.ascontiguousarray(pose13, np.float64))

    def add_edge(self, i, j, z13, info):
        rc = lib().lsdg_posegraph_add_edge(self._h, i, j, np.ascontiguousarray(z13, np.float64),
                                           np.ascontiguousarray(np.asarray(info, np.float64).reshape(49)))
        if rc != T.OK:
            raise LsdgError(rc, "lsdg_posegraph_add_edge")

    def optimize(self, iterations: int) -> float:
        c = C.c_double()
        lib().lsdg_posegraph_optimize(self._h, iterations, C.byref(c))
        return c.value

    def pose(self, i) -> np.ndarray:
        out = np.zeros(13)
        rc = lib().lsdg_posegraph_get_pose(self._h, i, out)
        if rc != T.OK:
            raise LsdgError(rc, "lsdg_posegraph_get_pose")
        return out

    def close(self):
        if self._h:
            lib().lsdg_posegraph_destroy(self._h)
            self._h = _vp()


def sim3_exp13(xi) -> np.ndarray:
    out = np.zeros(13)
    lib().lsdg_sim3_exp13(np.ascontiguousarray(xi, np.float64), out)
    return out


def sim3_log13(pose13) -> np.ndarray:
    out = np.zeros(7)
    lib().lsdg_sim3_log13(np.ascontiguousarray(pose13, np.float64), out)
    return out


def pack_pairs(pairs):
    """Concatenate synth.TrackingPair inputs into the back-to-back layout lsdg_batch_load expects."""
    cat = lambda name: np.ascontiguousarray(np.concatenate([getattr(q, name).ravel() for q in pairs]), np.float32)
    return cat("ref_image"), cat("ref_idepth"), cat("ref_idepth_var"), cat("new_image")


def pack_sim3_pairs(pairs):
    """Concatenate synth.Sim3Pair inputs into the layout lsdg_batch_load_sim3 expects."""
    cat = lambda name: np.ascontiguousarray(np.concatenate([getattr(q, name).ravel() for q in pairs]), np.float32)
    return (cat("ref_image"), cat("ref_idepth"), cat("ref_idepth_var"), cat("new_image"), cat("new_idepth"),
            cat("new_idepth_var"))


def declared_symbols(header: str = HEADER):
    """Names of the entry points include/lsdg.h declares."""
    import re
    txt = open(header).read()
    return sorted(set(re.findall(r"^LSDG_API\s+[\w\s\*]+?\b(lsdg_\w+)\s*\(", txt, flags=re.M)))
