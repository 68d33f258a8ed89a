"""ctypes mirrors of the plain-C structs declared in include/lsdg.h (no behaviour, layout only)."""
from __future__ import annotations

import ctypes as C

MAX_LEVELS = 6
NE_SIZE = 32
NE_SIZE_SIM3 = 40

OK = 0
INVALID_ARG = 1
TRACKING_LOST = 2
DIVERGED = 3
TIMEOUT = 4
CUDA_ERROR = 5
OUT_OF_MEMORY = 6
NOT_SUPPORTED = 7

STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "TRACKING_LOST", 3: "DIVERGED", 4: "TIMEOUT",
                5: "CUDA_ERROR", 6: "OUT_OF_MEMORY", 7: "NOT_SUPPORTED"}


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Params(C.Structure):
    _fields_ = [
        ("levels", C.c_int32),
        ("max_iterations", C.c_int32 * MAX_LEVELS),
        ("photometric_variance", C.c_float),
        ("huber_delta", C.c_float),
        ("min_z", C.c_float),
        ("border_margin", C.c_float),
        ("lm_lambda_initial", C.c_float),
        ("lm_lambda_up", C.c_float),
        ("lm_lambda_down", C.c_float),
        ("step_eps", C.c_float),
        ("stall_eps", C.c_float),
        ("min_good_ratio", C.c_float),
        ("min_usage", C.c_float),
        ("sim3_depth_variance", C.c_float),
        ("sim3_depth_weight", C.c_float),
        ("min_grad", C.c_float),
        ("min_idepth", C.c_float),
        ("max_idepth", C.c_float),
        ("epipolar_var", C.c_float),
        ("image_var", C.c_float),
        ("min_grad_along_epl2", C.c_float),
        ("max_ssd", C.c_float),
        ("unique_ratio", C.c_float),
        ("search_sigmas", C.c_float),
        ("max_search_len", C.c_float),
        ("min_search_len", C.c_float),
        ("fuse_chi2", C.c_float),
        ("min_epl_length", C.c_float),
        ("validity_init", C.c_int32),
        ("validity_max", C.c_int32),
        ("validity_penalty", C.c_int32),
        ("blacklist_limit", C.c_int32),
        ("prediction_var", C.c_float),
        ("propagate_max_photo_diff", C.c_float),
        ("reg_radius", C.c_int32),
        ("reg_chi2", C.c_float),
        ("reg_min_support", C.c_int32),
        ("fill_min_support", C.c_int32),
        ("fill_var_factor", C.c_float),
        ("refine_prior_weight", C.c_float),
        ("reserved", C.c_int32 * 7),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_bytes(self) -> bytes:
        return bytes(C.string_at(C.byref(self), C.sizeof(Params)))


class TrackStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("passes", C.c_int32 * MAX_LEVELS),
        ("total_passes", C.c_int32),
        ("n_points", C.c_int32),
        ("n_valid", C.c_int32),
        ("n_good", C.c_int32),
        ("mean_energy", C.c_float),
        ("good_ratio", C.c_float),
        ("usage", C.c_float),
        ("hessian", C.c_double * 28),
    ]

    def as_dict(self) -> dict:
        return {
            "status": STATUS_NAMES.get(self.status, str(self.status)),
            "passes": list(self.passes),
            "total_passes": self.total_passes,
            "n_points": self.n_points,
            "n_valid": self.n_valid,
            "n_good": self.n_good,
            "mean_energy": self.mean_energy,
            "good_ratio": self.good_ratio,
            "usage": self.usage,
        }


class CloudParams(C.Structure):
    """lsdg_cloud_params (include/lsdg.h)."""
    _fields_ = [("scaled_th", C.c_float), ("abs_th", C.c_float), ("min_near_support", C.c_int32),
                ("reserved", C.c_int32)]


CALIB_PINHOLE = 0
CALIB_FRAME = 1


class Calibration(C.Structure):
    """lsdg_calibration (include/lsdg.h)."""
    _fields_ = [("model", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("f", C.c_double), ("cx", C.c_double), ("cy", C.c_double), ("b1", C.c_double), ("b2", C.c_double),
                ("k1", C.c_double), ("k2", C.c_double), ("k3", C.c_double), ("k4", C.c_double),
                ("p1", C.c_double), ("p2", C.c_double)]


class SlamParams(C.Structure):
    """lsdg_slam_params (include/lsdg.h)."""
    _fields_ = [
        ("kf_dist", C.c_float), ("kf_angle_deg", C.c_float), ("kf_min_usage", C.c_float),
        ("refresh_every", C.c_int32), ("n_candidates", C.c_int32), ("cand_radius", C.c_float),
        ("optimize_every", C.c_int32), ("final_iterations", C.c_int32), ("max_track_jump", C.c_float),
        ("both_directions", C.c_int32), ("consistency_trans", C.c_float), ("consistency_rot", C.c_float),
        ("consistency_scale", C.c_float), ("async_constraints", C.c_int32), ("graph_threads", C.c_int32),
        ("odometry_scale_weight", C.c_float), ("ref_min_validity", C.c_int32), ("sim3_info_scale", C.c_float),
        ("ref_max_var", C.c_float), ("epipolar_var", C.c_float), ("reactivate", C.c_int32),
        ("react_radius", C.c_float), ("react_angle_deg", C.c_float), ("react_min_usage", C.c_float),
        ("react_max_jump", C.c_float), ("react_min_age", C.c_int32), ("react_min_good", C.c_float),
        ("retrack_iterations", C.c_int32), ("reserved", C.c_int32 * 1),
    ]


class SlamStats(C.Structure):
    """lsdg_slam_stats (include/lsdg.h)."""
    _fields_ = [("frames", C.c_int32), ("keyframes", C.c_int32), ("lost_frames", C.c_int32),
                ("sim3_edges", C.c_int32), ("sim3_rejected", C.c_int32), ("graph_optimisations", C.c_int32),
                ("reactivations", C.c_int32), ("reserved", C.c_int32 * 5)]


class GraphFramePose(C.Structure):
    """lsdg_graph_frame_pose: a keyframe id and the Sophus 7-float camToWorld (include/lsdg.h)."""
    _fields_ = [("id", C.c_int32), ("cam_to_world", C.c_float * 7)]

